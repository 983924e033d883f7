// crgpu_v1_body.cuh - device bodies of the v1 frontier kernels (see crgpu_v1.cu for the
// algorithm).  Each body runs on `nwk` workers (thread blocks) of which this block is `wk`:
// the stand-alone kernels pass (blockIdx.x, gridDim.x); the persistent batch kernel, where one
// block owns a whole solve, passes (0, 1) and separates the bodies with __syncthreads.
//
// The including file defines CR_BODY_NS (the namespace of this instance), CR_LDG (a load of
// data that does not change while the kernel runs), CR_RESTRICT and CR_BODY_INLINE.  Inside the persistent
// batch kernel a block writes the very buffers it later reads (and reuses them job after job),
// so there both are plain coherent loads; the stand-alone kernels use the read-only path.
#pragma once
#include "crgpu_internal.cuh"

namespace crgpu {
namespace CR_BODY_NS {


#define FULL_MASK 0xFFFFFFFFu
#define CR_MAX_K_DEV 4

// Lexicographic rank of a sorted multiset (see config_rank): B read through CR_LDG, or from
// shared memory when staged there.
template <int K>
__device__ __forceinline__ uint32_t rank_g(const int (&c)[K], const uint32_t* B, int np1) {
    uint32_t r = 0;
    int prev = 0;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        r += CR_LDG(&B[i * np1 + prev]) - CR_LDG(&B[i * np1 + c[i]]);
        prev = c[i];
    }
    return r;
}
template <int K>
__device__ __forceinline__ uint32_t rank_s(const int (&c)[K], const uint32_t* sB, int np1) {
    uint32_t r = 0;
    int prev = 0;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        r += sB[i * np1 + prev] - sB[i * np1 + c[i]];
        prev = c[i];
    }
    return r;
}

// Shared-memory words of one lane group of the last-column body.
__host__ __device__ inline int and_group_words(int S, int rwp) { return 3 * rwp + S * rwp; }

// Words of shared memory the pull body stages the rank table in (16-byte multiple).
__host__ __device__ inline int rank_table_words(int k, int n) { return (k * (n + 1) + 3) & ~3; }

// Words of shared memory the separable turn's pair rows stage frontier rows in (16 KB).
constexpr int kPairStageWords = 4096;

__device__ __forceinline__ bool frontier_sparse(const V1Dev& d, const ColMeta& m) {
    return (unsigned long long)m.rows * d.push_ratio < d.C;
}

// A warp's buffer of row ids bound for a column's list: up to 32 ids, one per lane, written out
// with one atomic on the list length when full and at the end (appends from every warp of a
// grid would otherwise serialise on that one counter, and a returning atomic per append puts
// its latency on the warp's path).
struct ListBuf {
    uint32_t lbuf = 0;
    int lcount = 0;   // warp-uniform

    __device__ __forceinline__ void spill(const V1Dev& d, int col, int lane) {
        int at = 0;
        if (lane == 0) at = atomicAdd(&d.meta[col].len, lcount);
        at = __shfl_sync(FULL_MASK, at, 0);
        if (lane < lcount) d.list[(size_t)col * d.C + at + lane] = lbuf;
        lcount = 0;
    }
    // Appends id for every lane whose pred is set (warp-collective).
    __device__ __forceinline__ void append(const V1Dev& d, int col, bool pred, uint32_t id, int lane) {
        const unsigned b = __ballot_sync(FULL_MASK, pred);
        if (!b) return;
        const int k = __popc(b);
        if (lcount + k > 32) spill(d, col, lane);
        // lane lcount + j takes the id of the j-th lane with pred set
        const bool dst = lane >= lcount && lane < lcount + k;
        const int src = dst ? (int)__fns(b, 0, lane - lcount + 1) : lane;
        const uint32_t v = __shfl_sync(FULL_MASK, id, src);
        if (dst) lbuf = v;
        lcount += k;
    }
    __device__ __forceinline__ void finish(const V1Dev& d, int col, int lane) {
        if (lcount) spill(d, col, lane);
    }
};

// Running totals of a producer (count of new marks, listed rows, value range, error bits) and
// its list buffer.  flush() empties the buffer and reduces the totals over the block, so a
// block reports with one atomic per field; every thread of the block calls it once, at the end
// of the body.
struct Tally {
    unsigned cnt = 0, err = 0, rows = 0;
    int lo = kEmptyLo, hi = -1;
    ListBuf lb;

    __device__ __forceinline__ void append(const V1Dev& d, int col, bool pred, uint32_t id, int lane) {
        lb.append(d, col, pred, id, lane);
    }
    __device__ void flush(const V1Dev& d, int col, int lane) {
        lb.finish(d, col, lane);
        __shared__ unsigned s_u[3][32];
        __shared__ int s_i[2][32];
        const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
        cnt = __reduce_add_sync(FULL_MASK, cnt);
        rows = __reduce_add_sync(FULL_MASK, rows);
        lo = __reduce_min_sync(FULL_MASK, lo);
        hi = __reduce_max_sync(FULL_MASK, hi);
        err = __reduce_or_sync(FULL_MASK, err);
        if (lane == 0) {
            s_u[0][w] = cnt;
            s_u[1][w] = rows;
            s_u[2][w] = err;
            s_i[0][w] = lo;
            s_i[1][w] = hi;
        }
        __syncthreads();
        if (w == 0) {
            const bool in = lane < nw;
            cnt = __reduce_add_sync(FULL_MASK, in ? s_u[0][lane] : 0u);
            rows = __reduce_add_sync(FULL_MASK, in ? s_u[1][lane] : 0u);
            err = __reduce_or_sync(FULL_MASK, in ? s_u[2][lane] : 0u);
            lo = __reduce_min_sync(FULL_MASK, in ? s_i[0][lane] : kEmptyLo);
            hi = __reduce_max_sync(FULL_MASK, in ? s_i[1][lane] : -1);
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
        __syncthreads();
    }
};

// Before a producer run of column `col` (whose inputs are column nx): clear the flags of the
// column's previous frontier unless its consumer already did (consumers that walk the row list
// clear each row's flag as they take it; the dense cop turns read flags at random and leave
// them), then fix the value base of the new frontier and empty its range and list -- unless
// the column is in append mode (column 0 in pass 1 after the unfused initializeCaptures, whose
// frontier already holds the capture seeds).  Before an odd column it also clears the candidate
// rows of the push-mode cop turn just run.  Every block reads the column's state first; the
// last block to finish (counted in sync[0]) resets it, so no block reads a half-reset state.
__device__ CR_BODY_INLINE void prep_clear_flags(const V1Dev& d, int col, unsigned wk, unsigned nwk) {
    const ColMeta* mo = d.meta + col;
    if (!mo->append && !mo->clean) {
        uint8_t* f = d.fflag + (size_t)col * d.C;
        for (size_t i = (size_t)wk * blockDim.x + threadIdx.x; i < d.C; i += (size_t)nwk * blockDim.x)
            f[i] = 0;
    }
}
// The candidate rows (and their bitmap words) the last push-mode cop turn consumed.
__device__ CR_BODY_INLINE void prep_clear_cand(const V1Dev& d, unsigned wk, unsigned nwk) {
    const size_t words = (size_t)d.S * d.g.rwp, total = (size_t)d.sync[1] * words;
    for (size_t i = (size_t)wk * blockDim.x + threadIdx.x; i < total; i += (size_t)nwk * blockDim.x) {
        const uint32_t cid = d.clist[i / words];
        const size_t e = i % words;
        d.cand[(size_t)cid * words + e] = 0u;
        if (e == 0) d.cbits[cid >> 5] = 0u;
    }
}
__device__ CR_BODY_INLINE void prep_clear(const V1Dev& d, int col, unsigned wk, unsigned nwk) {
    prep_clear_flags(d, col, wk, nwk);
    if (col % 2 == 1) prep_clear_cand(d, wk, nwk);
}

// Thread 0 of each block of a grid (after the block's work and a __syncthreads): true in the
// last block to arrive, counted in sync[0], which it resets.
__device__ __forceinline__ bool grid_last_block(const V1Dev& d, unsigned nwk) {
    bool last = nwk == 1;
    if (!last) {
        __threadfence();
        last = atomicAdd(&d.sync[0], 1u) == nwk - 1;
    }
    if (last) {
        __threadfence();
        if (nwk > 1) d.sync[0] = 0u;
    }
    return last;
}

// The column state reset of prep, done once (the last block).
__device__ CR_BODY_INLINE void prep_reset(const V1Dev& d, int col, int nx) {
    ColMeta* mo = d.meta + col;
    if (!mo->append) {
        const ColMeta mi = d.meta[nx];
        mo->old_hi = max(mo->old_hi, mo->hi);
        mo->base = (mi.hi >= mi.lo) ? mi.lo + 1 : 0;
        mo->lo = kEmptyLo;
        mo->hi = -1;
        mo->rows = 0;
        mo->len = 0;
        mo->clean = 0;
    }
    mo->seed = 0;
    if (col == 0) *d.pass_new = 0ull;
    if (col % 2 == 0) d.sync[1] = 0u;                // the push form's candidate list
    if (col == d.cols - 1) d.meta[0].append = 0;   // column 0's seeded frontier is consumed
}

__device__ CR_BODY_INLINE void prep_body(const V1Dev& d, int col, int nx, unsigned wk, unsigned nwk) {
    prep_clear(d, col, wk, nwk);
    __syncthreads();
    if (threadIdx.x == 0 && grid_last_block(d, nwk)) prep_reset(d, col, nx);
}

// The row list of a column's frontier as a consumer sees it: n entries, entry i = row id(i).
struct RowList {
    const uint32_t* ids;
    uint32_t n;
    bool all;
    __device__ RowList(const V1Dev& d, int col, const ColMeta& m)
        : ids(d.list + (size_t)col * d.C), n(m.len < 0 ? d.C : (uint32_t)m.len), all(m.len < 0) {}
    __device__ __forceinline__ uint32_t id(uint32_t i) const { return all ? i : CR_LDG(&ids[i]); }
};

// initializeCaptures (k_cops_visibility.cpp:85-127): the table was memset to 0xFE; a robber
// on a cop is a capture of round 0 in columns 0 and 1 only.  The seeds also form the first
// frontiers of columns 0 and 1 (value 0, slot 0); their rows are written whole.
__device__ CR_BODY_INLINE void init_body(const V1Dev& d, int K, unsigned wk, unsigned nwk) {
    unsigned caps = 0;
    const int n = d.g.n, rwp = d.g.rwp, S = d.S;
    for (uint32_t cid = wk * blockDim.x + threadIdx.x; cid < d.C;
         cid += nwk * blockDim.x) {
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

// 4 bits -> 4 bytes of 0xFF / 0x00 (bit i -> byte i).
__device__ __forceinline__ uint32_t nibble_bytes(uint32_t b) {
    return ((b * 0x00204081u) & 0x01010101u) * 0xFFu;
}

// Cover masks of 8 consecutive robbers (cover_w = W bytes each), packed in 2W words.
template <int W>
struct Cov8 {
    static constexpr int NW = 2 * W;
    uint32_t w[NW];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int q = 0; q < NW; ++q) w[q] = 0u;
    }
    __device__ __forceinline__ void load(const uint8_t* p) {   // p is 8W-byte aligned
        if (W == 1) {
            const uint2 v = CR_LDG(reinterpret_cast<const uint2*>(p));
            w[0] = v.x; w[1] = v.y;
        } else {
#pragma unroll
            for (int h = 0; h < W / 2; ++h) {
                const uint4 v = CR_LDG(reinterpret_cast<const uint4*>(p) + h);
                w[4 * h] = v.x; w[4 * h + 1] = v.y; w[4 * h + 2] = v.z; w[4 * h + 3] = v.w;
            }
        }
    }
    __device__ __forceinline__ void ones() {
#pragma unroll
        for (int q = 0; q < NW; ++q) w[q] = 0xFFFFFFFFu;
    }
    __device__ __forceinline__ void orr(const Cov8& o) {
#pragma unroll
        for (int q = 0; q < NW; ++q) w[q] |= o.w[q];
    }
    __device__ __forceinline__ void andd(const Cov8& o) {
#pragma unroll
        for (int q = 0; q < NW; ++q) w[q] &= o.w[q];
    }
    // some robber's mask is zero (the exact zero-byte / zero-halfword tests)
    __device__ __forceinline__ bool has_zero() const {
        uint32_t t = 0;
        if (W == 1) {
#pragma unroll
            for (int q = 0; q < 2; ++q) t |= (w[q] - 0x01010101u) & ~w[q] & 0x80808080u;
        } else if (W == 2) {
#pragma unroll
            for (int q = 0; q < 4; ++q) t |= (w[q] - 0x00010001u) & ~w[q] & 0x80008000u;
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) t |= w[q] == 0u ? 1u : 0u;
        }
        return t != 0u;
    }
    // bit j set iff robber j's mask is zero
    __device__ __forceinline__ uint32_t zero_bits() const {
        uint32_t b = 0;
        if (W == 1) {
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const uint32_t m = ~(((w[q] & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | w[q]) & 0x80808080u;
                b |= ((((m >> 7) & 0x01010101u) * 0x01020408u) >> 24) << (4 * q);
            }
        } else if (W == 2) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint32_t m = __vcmpeq2(w[q], 0u);
                b |= (((m >> 15) & 1u) | ((m >> 30) & 2u)) << (2 * q);
            }
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) b |= (uint32_t)(w[q] == 0u) << q;
        }
        return b;
    }
};

// The next sorted multiset in lexicographic order (the configuration order).
template <int K>
__device__ __forceinline__ void next_multiset(int (&c)[K], int n) {
    if (c[K - 1] < n - 1) {   // the common step: only the last cop moves on
        ++c[K - 1];
        return;
    }
    int i = 0;   // the rightmost position below n - 1 (registers only: no indexed access)
#pragma unroll
    for (int j = 1; j < K; ++j)
        if (c[j] < n - 1) i = j;
    int v = 0;
#pragma unroll
    for (int j = 0; j < K; ++j)
        if (j == i) v = c[j] + 1;
#pragma unroll
    for (int j = 0; j < K; ++j)
        if (j >= i) c[j] = v;
}

// initializeCaptures and the whole first pass of a p = 1 solve (two columns) in one sweep that
// writes every table byte once.  After initializeCaptures only the captures are marked (round
// 0, both columns), so the first pass has closed forms:
//   column 0 (cops to move, k_cops_visibility.cpp:160-197): a robber on N(cops) is caught by
//          one cop move when every cop can move -- round 1;
//   column 1 (robber to move, :235-288): a robber r off the cops is lost when every move lands
//          on a column-0 mark, N(r) within M0 = cops | N(cops) (cops alone when some cop cannot
//          move); its round is 1 + the largest column-0 round among N(r): 2 when some
//          neighbour is not a cop, else 1.
// With the uncovered-slot masks both tests are ANDs over the k cops: N(r) lies in M0 iff the
// AND of cover[c][r] (slots of r outside {c} + N(c)) is empty, and N(r) lies in the cops iff
// the AND of cover[n + c][r] (slots of r other than c) is empty.
// Column 1's marks form its output frontier (value base 1: slot 0 holds round 1, slot 1
// round 2).  Column 0's frontier is read only through its flags and range, and every
// configuration has captures, so every column-0 flag is set.
// Each warp sweeps a contiguous range of configurations, stepping the multiset itself, and
// keeps the masks of all cops but the last (they change once per n - c[k-2] steps).  Lane l
// owns robbers 8l .. 8l+7 of each 256-vertex block, i.e. one 16-byte piece of the row, and
// the 8-bit pieces of the marked and frontier rows, which four lanes assemble into a word.
// The caller sets meta[0] = {0, 0, 0, 0, C, 0}, meta[1] = {1, empty, -1, 0, 0, 0} and zeroes
// the pass counter; the pass counter then holds the first pass's count.  Column 0's list is the
// implicit one (every row); column 1's is built from its flags afterwards (list_compact), which
// keeps list atomics off the warps that own the rare column-1 rows.
// The same sweep for rows of one 256-robber block whose robbers split into whole lane pieces
// (n <= 256, n a multiple of 8), organised around the common configuration.  Consecutive
// configurations share their leading cops c[0 .. K-2] for a run of up to n of them (only the
// last cop moves on), so the sweep is a loop over runs and, inside, over the last cop.  What
// depends on the leading cops is set up once per run: the AND of their uncovered-slot masks,
// their neighbour word (column 0's marks are cops | N(cops)), their bits among the lane's
// robbers, and the 16-byte XOR patch that turns those robbers' bytes into 0x01 0x01.
// Per configuration the warp tests whether some robber of a lane is left with no uncovered slot
// (a zero mask after ANDing the last cop's cover row: one 8-byte load and a zero-byte test).
// The cover table is built so that this test also catches everything else the fast form does
// not handle: a cop's own entry cover[c][c] is all ones (a robber on a cop is a capture, never a
// column-1 mark, so the entry's value is otherwise irrelevant), and the rows of cops that cannot
// move are zero.  When no lane trips and every leading cop can move (nearly always), column 1
// gains no mark and the configuration takes the fast form: the lane's 16-byte piece is a
// shared-memory table entry indexed by its 8 column-0 seed bits, XORed with the leading cops'
// patch and stored once; the last cop's two bytes follow as one 2-byte store; one store per
// row word writes the marked words; nothing else is written (the column-1 frontier row stays
// unwritten and its flag clear: the warp sets its configurations' flag bytes first).  The fast
// form runs as a tight inner loop over per-lane cursors (piece, marked word, cover row,
// neighbour word, the last cop's offsets) and leaves it only for a configuration that trips,
// which takes the general form: every robber tested exactly, the column-1 marks split by round,
// their bytes patched and the frontier words written.  FULL (n = 256) lets every lane own eight
// robbers, which removes the lane predicates.  Results are byte-identical to the general sweep.
// Dynamic shared memory: init_pass1_smem_words(n, rwp) words.
__host__ __device__ inline int init_pass1_smem_words(int n, int rwp) { return 256 * 4 + n * rwp; }

template <int K, int W, bool FULL>
__device__ CR_BODY_INLINE void init_pass1_single(const V1Dev& d, unsigned wk, unsigned nwk) {
    extern __shared__ uint32_t sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // FULL: n = 256 exactly, so every lane owns 8 robbers and every row word has a lane
    const int n = FULL ? 256 : d.g.n, rw = FULL ? 8 : d.g.rw, rwp = FULL ? 8 : d.g.rwp;
    const int S = d.S, npad = FULL ? 256 : d.g.npad;
    const uint32_t C = d.C;
    const uint32_t* CR_RESTRICT iso = cop_iso(d.g);
    const uint8_t* CR_RESTRICT cover = d.g.cover;
    uint8_t* const table = d.table;
    uint32_t* const marked = d.marked;
    const size_t plane = (size_t)n * npad * W;
    const bool padded = rw != rwp || S > 2;
    // shared memory: the piece table (entry s: robbers j with bit j of s set read 0x03 in
    // column 0, every other byte 0xFE) and the cops' neighbour rows
    uint4* lut = reinterpret_cast<uint4*>(sm);
    uint32_t* snbr = sm + 256 * 4;
    for (int t = threadIdx.x; t < 256; t += blockDim.x) {
        const uint32_t s0 = 0xFEFEFEFEu ^ (nibble_bytes(t & 0xF) & 0xFDFDFDFDu);
        const uint32_t s1 = 0xFEFEFEFEu ^ (nibble_bytes(t >> 4) & 0xFDFDFDFDu);
        const uint32_t fe = 0xFEFEFEFEu;
        lut[t] = make_uint4(__byte_perm(s0, fe, 0x5140), __byte_perm(s0, fe, 0x7362),
                            __byte_perm(s1, fe, 0x5140), __byte_perm(s1, fe, 0x7362));
    }
    for (int t = threadIdx.x; t < n * rwp; t += blockDim.x) snbr[t] = CR_LDG(&d.g.nbr[t]);
    __syncthreads();
    unsigned cnt = 0, cnt1 = 0, rows1 = 0, any1 = 0, any2 = 0;
    const size_t nwarps = (size_t)nwk * (blockDim.x >> 5);
    const size_t chunk = (C + nwarps - 1) / nwarps;
    const size_t cb = ((size_t)wk * (blockDim.x >> 5) + warp) * chunk;
    const size_t ce = cb + chunk < C ? cb + chunk : C;
    int c[K];
    if (cb < ce) {
#pragma unroll
        for (int i = 0; i < K; ++i) c[i] = CR_LDG(&d.configs[cb * K + i]);
    }
    const int lr0 = lane * 8;                 // this lane's robbers lr0 .. lr0 + 7
    const bool live = FULL || lr0 < n;
    const int wi = lane >> 2;                 // their word of a robber row
    const int sh = (lane & 3) * 8;            // and their bit offset in it
    const uint32_t lvalid = live ? 0xFFu : 0u;
    const bool writer = (lane & 3) == 0 && (FULL || wi < rw);
    // fast form: lane 4w writes word w of the column-0 marked row, lane 4w + 1 that of column 1
    const bool mwriter = (lane & 3) < 2 && (FULL || wi < rw);
    const size_t mplane = (lane & 1) ? (size_t)C * rwp : 0;
    // the flag planes of this warp's configurations: column 0 clear (its frontier, every row,
    // is consumed by the last column fused here, so the column starts pass 2 clean), column 1
    // clear (set below for the rows that gain marks)
    for (size_t i = cb + lane; i < ce; i += 32) {
        d.fflag[i] = 0;
        d.fflag[(size_t)C + i] = 0;
    }
    __syncwarp();
    size_t cid = cb;
    while (cid < ce) {
        // a new run of the leading cops c[0 .. K-2]: the AND of their uncovered masks (with and
        // without their neighbourhoods), whether all can move, their neighbour word, their bits
        // among this lane's robbers and in its word, and the XOR patch of their bytes
        Cov8<W> zpre, znpre;
        zpre.ones();
        znpre.ones();
        bool mpre = true;
        uint32_t npre = 0, cpre = 0, cpw = 0;
#pragma unroll
        for (int i = 0; i < K - 1; ++i) {
            mpre &= !((CR_LDG(&iso[c[i] >> 5]) >> (c[i] & 31)) & 1u);
            if ((c[i] >> 5) == wi) cpw |= 1u << (c[i] & 31);
            if (live) {
                npre |= snbr[c[i] * rwp + wi];
                const unsigned dv = (unsigned)(c[i] - lr0);
                if (dv < 8u) cpre |= 1u << dv;
                Cov8<W> t;
                t.load(cover + (uint32_t)(c[i] * npad + lr0) * W);
                zpre.andd(t);
                t.load(cover + plane + (uint32_t)(c[i] * npad + lr0) * W);
                znpre.andd(t);
            }
        }
        uint4 capx;
        capx.x = ((cpre & 1u) ? 0x0000FFFFu : 0u) | ((cpre & 2u) ? 0xFFFF0000u : 0u);
        capx.y = ((cpre & 4u) ? 0x0000FFFFu : 0u) | ((cpre & 8u) ? 0xFFFF0000u : 0u);
        capx.z = ((cpre & 16u) ? 0x0000FFFFu : 0u) | ((cpre & 32u) ? 0xFFFF0000u : 0u);
        capx.w = ((cpre & 64u) ? 0x0000FFFFu : 0u) | ((cpre & 128u) ? 0xFFFF0000u : 0u);
        const int cl0 = c[K - 1];
        const size_t cid0 = cid;
        const uint32_t len = (uint32_t)(cid0 + (size_t)(n - cl0) < ce ? (size_t)(n - cl0) : ce - cid0);
        cid += len;
        // per-lane cursors of the run: the lane's piece, its marked word, its cover row (lanes
        // without robbers read lane 0's), its neighbour word, the last cop's offset from the
        // lane's robbers and from its row word
        uint8_t* dst = table + cid0 * n * 2 + lr0 * 2;
        uint32_t* mrow = marked + mplane + cid0 * rwp + wi;
        const uint8_t* cv = cover + (size_t)(cl0 * npad + (live ? lr0 : 0)) * W;
        const uint32_t* nb = snbr + cl0 * rwp + (live ? wi : 0);
        int dl = cl0 - lr0, dw = cl0 - 32 * wi;
        uint32_t j = 0;
        while (j < len) {
            // fast form while every cop can move and column 1 gains no mark
            for (; j < len; ++j, dst += 2 * n, mrow += rwp, cv += npad * W, nb += rwp, ++dl, ++dw) {
                Cov8<W> z;
                z.load(cv);
                z.andd(zpre);
                if (__any_sync(FULL_MASK, live && z.has_zero()) || !mpre) break;
                const uint32_t c2b = (unsigned)dl < 8u ? 1u << dl : 0u;
                const uint32_t capw = cpw | ((unsigned)dw < 32u ? 1u << dw : 0u);
                const uint32_t xw = npre | *nb;
                const uint32_t seedb = (xw >> sh) & lvalid & ~(cpre | c2b);
                uint4 pc = lut[seedb];
                pc.x ^= capx.x;
                pc.y ^= capx.y;
                pc.z ^= capx.z;
                pc.w ^= capx.w;
                if (live) *reinterpret_cast<uint4*>(dst) = pc;
                if (c2b) *reinterpret_cast<uint16_t*>(dst + 2 * dl) = 0x0101u;
                cnt += __popc(seedb);
                if (mwriter) *mrow = (lane & 1) ? capw : (xw | capw);
                if (padded) {
                    uint32_t* m0row = marked + (cid0 + j) * rwp;
                    uint32_t* m1row = marked + ((size_t)C + cid0 + j) * rwp;
                    for (int e = rw + lane; e < rwp; e += 32) {
                        m0row[e] = 0u;
                        m1row[e] = 0u;
                    }
                }
            }
            if (j >= len) break;
            // general form of configuration cid0 + j
            const int cl = cl0 + (int)j;
            const size_t id = cid0 + j;
            const unsigned dlu = (unsigned)dl;
            const uint32_t capb = cpre | (dlu < 8u ? 1u << dlu : 0u);
            const uint32_t capw = cpw | ((unsigned)dw < 32u ? 1u << dw : 0u);
            const bool moves = mpre && !((CR_LDG(&iso[cl >> 5]) >> (cl & 31)) & 1u);
            const uint32_t off = (uint32_t)(cl * npad + lr0) * W;
            uint32_t xw = 0, a = 0;
            if (live) {
                // N(r) within M0 iff no slot of r stays uncovered (M0 = the cops alone when
                // some cop cannot move)
                Cov8<W> z = moves ? zpre : znpre, t;
                t.load(cover + (moves ? 0 : plane) + off);
                z.andd(t);
                a = z.zero_bits() & ~capb & lvalid;
                if (moves) xw = npre | snbr[cl * rwp + wi];
            }
            const uint32_t seedb = (xw >> sh) & 0xFFu & ~capb;
            if (live) {
                uint4 pc = lut[seedb];
                pc.x ^= capx.x;
                pc.y ^= capx.y;
                pc.z ^= capx.z;
                pc.w ^= capx.w;
                *reinterpret_cast<uint4*>(dst) = pc;
                if (dlu < 8u) *reinterpret_cast<uint16_t*>(dst + 2 * dlu) = 0x0101u;
            }
            cnt += __popc(seedb);
            uint32_t m1w = capw;
            const bool changed = __any_sync(FULL_MASK, a != 0u);
            if (changed) {
                // column-1 marks: round 2 when some neighbour of r is not a cop, else round 1
                uint32_t deepb = 0;
                if (live) {
                    Cov8<W> zn = znpre, t;
                    t.load(cover + plane + off);
                    zn.andd(t);
                    deepb = ~zn.zero_bits();
                }
                const uint32_t a2 = a & deepb, a1 = a & ~deepb;
                uint32_t sp = a;
                while (sp) {
                    const int jb = __ffs(sp) - 1;
                    sp &= sp - 1;
                    const uint32_t bit = 1u << jb;
                    const uint32_t v0 = (seedb & bit) ? 0x03u : 0xFEu;
                    const uint32_t v1 = (a1 & bit) ? 0x03u : 0x05u;
                    *reinterpret_cast<uint16_t*>(dst + 2 * jb) = (uint16_t)(v0 | (v1 << 8));
                }
                cnt1 += __popc(a1) + __popc(a2);
                any1 |= a1;
                any2 |= a2;
                // the 8-bit pieces of lanes 4w .. 4w+3 make word w of the column-1 frontier slots
                const uint32_t v = a1 | a2 << 8;
                const uint32_t v1 = __shfl_down_sync(FULL_MASK, v, 1);
                const uint32_t v2 = __shfl_down_sync(FULL_MASK, v, 2);
                const uint32_t v3 = __shfl_down_sync(FULL_MASK, v, 3);
                const uint32_t t01 = __byte_perm(v, v1, 0x5140), t23 = __byte_perm(v2, v3, 0x5140);
                const uint32_t a1w = __byte_perm(t01, t23, 0x5410), a2w = __byte_perm(t01, t23, 0x7632);
                m1w |= a1w | a2w;
                uint32_t* frow = d.front + ((size_t)C + id) * (size_t)(S * rwp);
                if (writer) {
                    frow[wi] = a1w;
                    frow[rwp + wi] = a2w;
                }
                if (padded) {
                    for (int e = rw + lane; e < rwp; e += 32) {
                        frow[e] = 0u;
                        frow[rwp + e] = 0u;
                    }
                    for (int e = 2 * rwp + lane; e < S * rwp; e += 32) frow[e] = 0u;
                }
                if (lane == 0) {
                    d.fflag[(size_t)C + id] = 1;
                    ++rows1;
                }
            }
            uint32_t* m0row = marked + id * rwp;
            uint32_t* m1row = marked + ((size_t)C + id) * rwp;
            if (writer) {
                m0row[wi] = xw | capw;
                m1row[wi] = m1w;
            }
            if (padded) {
                for (int e = rw + lane; e < rwp; e += 32) {
                    m0row[e] = 0u;
                    m1row[e] = 0u;
                }
            }
            ++j;
            dst += 2 * n;
            mrow += rwp;
            cv += npad * W;
            nb += rwp;
            ++dl;
            ++dw;
        }
        // the run is over: step the multiset past its last configuration
        if (cid < ce) {
            c[K - 1] = n - 1;
            next_multiset<K>(c, n);
        }
    }
    const unsigned seeds = __reduce_add_sync(FULL_MASK, cnt);
    cnt1 = __reduce_add_sync(FULL_MASK, cnt1);
    rows1 = __reduce_add_sync(FULL_MASK, rows1);
    any1 = __reduce_or_sync(FULL_MASK, any1);
    any2 = __reduce_or_sync(FULL_MASK, any2);
    if (lane == 0) {
        if (seeds + cnt1) atomicAdd(d.pass_new, (unsigned long long)(seeds + cnt1));
        if (rows1) atomicAdd(&d.meta[1].rows, (int)rows1);
        if (seeds) atomicMax(&d.meta[0].hi, 1);
        if (any1 | any2) {
            atomicMin(&d.meta[1].lo, any1 ? 1 : 2);
            atomicMax(&d.meta[1].hi, any2 ? 2 : 1);
        }
    }
}

// The general sweep (any row shape; the launcher sends single-block rows of whole lane pieces
// to init_pass1_single).
template <int K, int W>
__device__ CR_BODY_INLINE void init_pass1_body(const V1Dev& d, unsigned wk, unsigned nwk) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = d.g.n, rw = d.g.rw, rwp = d.g.rwp, S = d.S, npad = d.g.npad;
    const uint32_t* CR_RESTRICT nbr = d.g.nbr;
    const uint32_t* CR_RESTRICT iso = cop_iso(d.g);     // cops that cannot move
    const uint8_t* CR_RESTRICT cover = d.g.cover;
    const size_t plane = (size_t)n * npad * W;          // bytes of one cover plane
    const bool aligned = (n & 7) == 0, single = n <= 256;
    const bool padded = rw != rwp || S > 2;             // row words beyond the marks to clear
    unsigned cnt = 0, rows1 = 0, any_seed = 0, any1 = 0, any2 = 0;
    const size_t nwarps = (size_t)nwk * (blockDim.x >> 5);
    const size_t chunk = (d.C + nwarps - 1) / nwarps;
    const size_t cb = ((size_t)wk * (blockDim.x >> 5) + warp) * chunk;
    const size_t ce = cb + chunk < d.C ? cb + chunk : d.C;
    int c[K];
    if (cb < ce) {
#pragma unroll
        for (int i = 0; i < K; ++i) c[i] = CR_LDG(&d.configs[cb * K + i]);
    }
    // state of the cops c[0 .. K-2], kept while they stay put (single-block rows only):
    // AND of their uncovered masks, their out-neighbours (word lane/4), their bits among this
    // lane's robbers, and whether all of them can move
    int pre[K > 1 ? K - 1 : 1];
#pragma unroll
    for (int i = 0; i < K - 1; ++i) pre[i] = -1;
    Cov8<W> zpre, znpre;
    bool mpre = true;
    uint32_t npre = 0, cpre = 0;
    zpre.ones();
    znpre.ones();
    const int lr0 = lane * 8;                            // this lane's robbers in block 0
    const uint32_t lvalid = n - lr0 >= 8 ? 0xFFu : (lr0 < n ? (1u << (n - lr0)) - 1u : 0u);
    // row pointers advanced per configuration (no per-row index arithmetic)
    uint8_t* trow = d.table + cb * n * 2;
    uint32_t* m0row = d.marked + cb * rwp;
    uint32_t* m1row = d.marked + ((size_t)d.C + cb) * rwp;
    const int frow_words = S * rwp;
    uint32_t* frow = d.front + ((size_t)d.C + cb) * frow_words;
    uint8_t* fl0 = d.fflag + cb;
    uint8_t* fl1 = d.fflag + (size_t)d.C + cb;
    for (size_t cid = cb; cid < ce; ++cid, trow += 2 * n, m0row += rwp, m1row += rwp, frow += frow_words,
                ++fl0, ++fl1) {
        if (cid > cb) next_multiset<K>(c, n);
        const int cl = c[K - 1];
        bool same = true;
#pragma unroll
        for (int i = 0; i < K - 1; ++i) same &= pre[i] == c[i];
        if (!same) {
            // the leading cops moved: rebuild their state
            zpre.ones();
            znpre.ones();
            mpre = true;
            npre = 0;
            cpre = 0;
#pragma unroll
            for (int i = 0; i < K - 1; ++i) {
                pre[i] = c[i];
                mpre &= !((CR_LDG(&iso[c[i] >> 5]) >> (c[i] & 31)) & 1u);
                if (single && lr0 < n) {
                    npre |= CR_LDG(&nbr[c[i] * rwp + (lane >> 2)]);
                    const unsigned dv = (unsigned)(c[i] - lr0);
                    if (dv < 8u) cpre |= 1u << dv;
                    Cov8<W> t;
                    t.load(cover + (uint32_t)(c[i] * npad + lr0) * W);
                    zpre.andd(t);
                    t.load(cover + plane + (uint32_t)(c[i] * npad + lr0) * W);
                    znpre.andd(t);
                }
            }
        }
        const bool moves = mpre && !((CR_LDG(&iso[cl >> 5]) >> (cl & 31)) & 1u);
        bool changed = false;
        for (int r0 = lr0, it = 0; it * 256 < n; r0 += 256, ++it) {
            uint32_t capb = 0, seedb = 0, a1 = 0, a2 = 0;
            if (r0 < n) {
                const int wi = r0 >> 5;
                uint32_t xw = 0, validb = lvalid;
                Cov8<W> z, zn, t;
                const uint32_t off = (uint32_t)(cl * npad + r0) * W;
                if (single) {
                    const unsigned dv = (unsigned)(cl - r0);
                    capb = cpre | (dv < 8u ? 1u << dv : 0u);
                    if (moves) xw = npre | CR_LDG(&nbr[cl * rwp + wi]);
                    z = zpre;
                    zn = znpre;
                } else {
                    validb = n - r0 >= 8 ? 0xFFu : ((1u << (n - r0)) - 1u);
#pragma unroll
                    for (int i = 0; i < K; ++i) {
                        const unsigned dv = (unsigned)(c[i] - r0);
                        if (dv < 8u) capb |= 1u << dv;
                        if (moves) xw |= CR_LDG(&nbr[c[i] * rwp + wi]);
                    }
                    z.ones();
                    zn.ones();
#pragma unroll
                    for (int i = 0; i < K - 1; ++i) {
                        t.load(cover + (uint32_t)(c[i] * npad + r0) * W);
                        z.andd(t);
                        t.load(cover + plane + (uint32_t)(c[i] * npad + r0) * W);
                        zn.andd(t);
                    }
                }
                seedb = (xw >> (r0 & 31)) & 0xFFu & ~capb;
                t.load(cover + plane + off);
                zn.andd(t);
                if (moves) {
                    t.load(cover + off);
                    z.andd(t);
                } else {
                    z = zn;
                }
                // every slot of r in M0 (comp) / some slot of r not a cop (deep)
                const uint32_t a = z.zero_bits() & ~capb & validb;
                const uint32_t deepb = ~zn.zero_bits();
                a2 = a & deepb;
                a1 = a & ~deepb;
                // the piece: column 0 = 0x03 on the seeds (0xFE ^ 0xFD), else 0xFE; column 1 =
                // 0xFE; state (r, col) is byte 2r + col of the row.  The few cops and column-1
                // marks get their two bytes rewritten after the piece, in this thread's order.
                uint8_t* dst = trow + r0 * 2;
                const uint32_t s0 = 0xFEFEFEFEu ^ (nibble_bytes(seedb & 0xFu) & 0xFDFDFDFDu);
                const uint32_t s1 = 0xFEFEFEFEu ^ (nibble_bytes(seedb >> 4) & 0xFDFDFDFDu);
                const uint32_t fe = 0xFEFEFEFEu;
                if (aligned) {
                    *reinterpret_cast<uint4*>(dst) = make_uint4(__byte_perm(s0, fe, 0x5140), __byte_perm(s0, fe, 0x7362),
                                                                __byte_perm(s1, fe, 0x5140), __byte_perm(s1, fe, 0x7362));
                } else {
                    for (int b = 0; b < 16 && r0 + (b >> 1) < n; ++b)
                        dst[b] = (b & 1) ? 0xFE : (((seedb >> (b >> 1)) & 1u) ? 0x03 : 0xFE);
                }
                uint32_t special = capb | a1 | a2;
                while (special) {
                    const int j = __ffs(special) - 1;
                    special &= special - 1;
                    const uint32_t bit = 1u << j;
                    // column 0: 0x01 cop / 0x03 seed / 0xFE; column 1: 0x01 cop / 0x03 round 1 /
                    // 0x05 round 2 / 0xFE
                    const uint32_t v0 = (capb & bit) ? 0x01u : ((seedb & bit) ? 0x03u : 0xFEu);
                    const uint32_t v1 = (capb & bit) ? 0x01u : ((a1 & bit) ? 0x03u : ((a2 & bit) ? 0x05u : 0xFEu));
                    *reinterpret_cast<uint16_t*>(dst + 2 * j) = (uint16_t)(v0 | (v1 << 8));
                }
                cnt += __popc(seedb) + __popc(a1) + __popc(a2);
                any_seed |= seedb;
                any1 |= a1;
                any2 |= a2;
            }
            // the 8-bit pieces of four lanes make one word of each row: column-0 marks,
            // column-1 marks, column-1 frontier slots 0 and 1
            const uint32_t v = (capb | seedb) | (capb | a1 | a2) << 8 | a1 << 16 | a2 << 24;
            const uint32_t v1 = __shfl_down_sync(FULL_MASK, v, 1);
            const uint32_t v2 = __shfl_down_sync(FULL_MASK, v, 2);
            const uint32_t v3 = __shfl_down_sync(FULL_MASK, v, 3);
            const uint32_t t01 = __byte_perm(v, v1, 0x5140), t01b = __byte_perm(v, v1, 0x7362);
            const uint32_t t23 = __byte_perm(v2, v3, 0x5140), t23b = __byte_perm(v2, v3, 0x7362);
            const int w = it * 8 + (lane >> 2);
            const bool writer = (lane & 3) == 0 && w < rw;
            if (writer) {
                m0row[w] = __byte_perm(t01, t23, 0x5410);
                m1row[w] = __byte_perm(t01, t23, 0x7632);
            }
            // the frontier row is read only under its flag: a one-block row is written only
            // when it changed (longer rows always, as a later block may set the flag)
            const bool marks = __any_sync(FULL_MASK, (a1 | a2) != 0u);
            changed |= marks;
            if (marks || !single) {
                if (writer) {
                    frow[w] = __byte_perm(t01b, t23b, 0x5410);
                    frow[rwp + w] = __byte_perm(t01b, t23b, 0x7632);
                }
            }
        }
        if (padded) {
            for (int e = rw + lane; e < rwp; e += 32) {
                m0row[e] = 0u;
                m1row[e] = 0u;
                frow[e] = 0u;
                frow[rwp + e] = 0u;
            }
            for (int e = 2 * rwp + lane; e < frow_words; e += 32) frow[e] = 0u;
        }
        if (lane == 0) {
            *fl0 = 0;   // column 0's frontier is consumed here (the fused last column)
            *fl1 = changed ? 1 : 0;
            rows1 += changed ? 1u : 0u;
        }
    }
    cnt = __reduce_add_sync(FULL_MASK, cnt);
    rows1 = __reduce_add_sync(FULL_MASK, rows1);
    any_seed = __reduce_or_sync(FULL_MASK, any_seed);
    any1 = __reduce_or_sync(FULL_MASK, any1);
    any2 = __reduce_or_sync(FULL_MASK, any2);
    if (lane == 0) {
        if (cnt) atomicAdd(d.pass_new, (unsigned long long)cnt);
        if (rows1) atomicAdd(&d.meta[1].rows, (int)rows1);
        if (any_seed) atomicMax(&d.meta[0].hi, 1);
        if (any1 | any2) {
            atomicMin(&d.meta[1].lo, any1 ? 1 : 2);
            atomicMax(&d.meta[1].hi, any2 ? 2 : 1);
        }
    }
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
    const bool newrow = L.any(any != 0);
    if (newrow) {
        if (gl < rw) {
            d.marked[((size_t)col * d.C + cid) * rwp + gl] = mm;
            t.cnt += __popc(mm ^ m);
        }
        {
            uint32_t* frow = d.front + ((size_t)col * d.C + cid) * S * rwp;
            for (int e = gl; e < S * rwp; e += G) {
                const int so = e / rwp, w = e - so * rwp;
                const int s = out_base + so - base_in - 1;
                const uint32_t val = (s >= 0 && s < s_used && w < rw) ? wnew[s * rwp + w] : 0u;
                frow[e] = append ? (frow[e] | val) : val;
            }
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
    // (in append mode every row is already listed: the list is the implicit one)
    t.append(d, col, newrow && gl == 0 && !append, cid, L.lane);
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
__device__ CR_BODY_INLINE void cop_pull_body(const V1Dev& d, int col, int nx, unsigned wk, unsigned nwk) {
    extern __shared__ uint32_t sm[];
    constexpr int CPW = 32 / G;
    constexpr int U = 4;  // successor tuples in flight per lane
    const int warp = threadIdx.x >> 5;
    const Lanes<G> L(threadIdx.x & 31);
    const int gl = L.glane;
    const int n = d.g.n, rw = d.g.rw, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (mi.hi < mi.lo) return;                              // empty frontier: nothing changes
    if (mi.seed || frontier_sparse(d, mi)) return;       // the seed or push form handles it
    if (K == 3 && d.h1) return;                             // the separable form handles it
    const int base_in = mi.base;
    const int s_used = min(mi.hi - base_in + 1, S);
    const int nwords = s_used * rwp;
    const int out_base = d.meta[col].base;
    const int append = d.meta[col].append;
    const int np1 = n + 1;
    // the rank table lives in shared memory for the whole body
    uint32_t* sB = sm;
    for (int i = threadIdx.x; i < K * np1; i += blockDim.x) sB[i] = CR_LDG(&d.binom[i]);
    __syncthreads();
    uint32_t* wacc = sm + rank_table_words(K, n) + (warp * CPW + L.grp) * (2 * S * rwp);
    uint32_t* wnew = wacc + S * rwp;
    const uint32_t* CR_RESTRICT fin = d.front + (size_t)nx * d.C * S * rwp;
    const uint8_t* CR_RESTRICT fflag_in = d.fflag + (size_t)nx * d.C;
    const uint32_t* CR_RESTRICT rp = cop_rows(d.g);     // the cops' moves
    const uint16_t* CR_RESTRICT adj = cop_cols(d.g);
    const bool vec4 = (rwp & 3) == 0;
    const bool spec = (unsigned long long)mi.rows * 2 >= d.C;   // at least half the rows flagged
    Tally t;
    const size_t step = (size_t)nwk * (blockDim.x >> 5) * CPW;
    for (size_t cb = ((size_t)wk * (blockDim.x >> 5) + warp) * CPW; cb < d.C; cb += step) {
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
                lo[i] = CR_LDG(&rp[v]);
                dg[i] = CR_LDG(&rp[v + 1]) - lo[i];
                T *= dg[i];
            }
        }
        {
            uint32_t acc[NWP];
#pragma unroll
            for (int i = 0; i < NWP; ++i) acc[i] = 0u;
            const int Tmax = __reduce_max_sync(FULL_MASK, T);
            // odometer over N(c_0) x ... x N(c_{K-1}), last index fastest: this lane starts at
            // tuple gl and steps by G (one division per configuration, not per tuple)
            int idx[K];
            {
                int rem = T > 0 ? gl : 0;
#pragma unroll
                for (int i = K - 1; i >= 0; --i) {
                    const int q = dg[i] > 0 ? rem / dg[i] : 0;
                    idx[i] = rem - q * dg[i];
                    rem = q;
                }
            }
            for (int t0 = 0; t0 < Tmax; t0 += G * U) {
                uint32_t s[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    s[u] = 0xFFFFFFFFu;
                    if (t0 + u * G + gl < T) {
                        int c[K];
#pragma unroll
                        for (int i = 0; i < K; ++i) c[i] = CR_LDG(&adj[lo[i] + idx[i]]);
                        sort_small<K>(c);
                        s[u] = rank_s<K>(c, sB, np1);
                        int carry = G;
#pragma unroll
                        for (int i = K - 1; i >= 0; --i) {
                            if (!carry) break;
                            const int v = idx[i] + carry;
                            if (i == 0 || v < dg[i]) { idx[i] = v; carry = 0; }
                            else if (v < 2 * dg[i]) { idx[i] = v - dg[i]; carry = 1; }
                            else { carry = v / dg[i]; idx[i] = v - carry * dg[i]; }
                        }
                    }
                }
                unsigned ok = 0;
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (s[u] == 0xFFFFFFFFu) continue;
                    if (s[u] >= d.C) { t.err |= kErrRank; continue; }
                    ok |= 1u << u;
                }
                if (spec) {
                    // most rows are flagged: load flag and row together (one round trip), keep
                    // the row only if flagged (unflagged rows hold stale marks)
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (!((ok >> u) & 1u)) continue;
                        const uint32_t keep = CR_LDG(&fflag_in[s[u]]) ? 0xFFFFFFFFu : 0u;
                        const uint32_t* row = fin + (size_t)s[u] * S * rwp;
                        if (vec4) {
#pragma unroll
                            for (int w = 0; w < NWP; w += 4) {
                                if (w < nwords) {
                                    const uint4 x = CR_LDG(reinterpret_cast<const uint4*>(row + w));
                                    acc[w] |= x.x & keep; acc[w + 1] |= x.y & keep;
                                    acc[w + 2] |= x.z & keep; acc[w + 3] |= x.w & keep;
                                }
                            }
                        } else {
#pragma unroll
                            for (int w = 0; w < NWP; ++w)
                                if (w < nwords) acc[w] |= CR_LDG(row + w) & keep;
                        }
                    }
                    continue;
                }
                unsigned live = 0;
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (((ok >> u) & 1u) && CR_LDG(&fflag_in[s[u]])) live |= 1u << u;
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (!((live >> u) & 1u)) continue;
                    const uint32_t* row = fin + (size_t)s[u] * S * rwp;
                    if (vec4) {
#pragma unroll
                        for (int w = 0; w < NWP; w += 4) {
                            if (w < nwords) {
                                const uint4 x = CR_LDG(reinterpret_cast<const uint4*>(row + w));
                                acc[w] |= x.x; acc[w + 1] |= x.y; acc[w + 2] |= x.z; acc[w + 3] |= x.w;
                            }
                        }
                    } else {
#pragma unroll
                        for (int w = 0; w < NWP; ++w)
                            if (w < nwords) acc[w] |= CR_LDG(row + w);
                    }
                }
            }
            group_or<NWP, G>(acc, gl, wacc, need ? nwords : 0);
        }
        __syncwarp();
        emit_row<G>(d, cid, need, col, m, wacc, wnew, base_in, s_used, out_base, append, L, t);
    }
    t.flush(d, col, L.lane);
}

// Pair index of the multiset {x <= y} among all pairs in lexicographic order, and its inverse.
__device__ __forceinline__ uint32_t pair_index(int x, int y, int n) {
    return (uint32_t)(x * (2 * n - x + 1) / 2 + (y - x));
}
__device__ __forceinline__ void pair_of(uint32_t q, int n, int& x, int& y) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((uint32_t)(mid * (2 * n - mid + 1) / 2) <= q) lo = mid;
        else hi = mid - 1;
    }
    x = lo;
    y = lo + (int)(q - (uint32_t)(lo * (2 * n - lo + 1) / 2));
}

// Dense cop turn for k = 3 in separable form.  The OR over T(C) of the frontier rows F[C'],
// C' = sort(x, y, z) with x in N(c1), y in N(c2), z in N(c3), splits into two stages:
//   H1[{x, y}][c] = OR over z in N(c) of F[sort(x, y, z)]             (pair_h1_body)
//   acc(C)        = OR over x in N(c1), y in N(c2) of H1[{x, y}][c3]  (sep_pull_body)
// so a configuration reads deg^2 rows of H1 (consecutive configurations read consecutive
// rows) instead of ranking and gathering deg^3 successor tuples.  OR is exact, so the marks
// are the pull's.
// Stage 1: a block per pair {x, y}.  Its n frontier rows F[sort(x, y, z)], z = 0 .. n-1, are
// staged in shared memory (one rank and one row load per z; a row whose flag is clear counts
// as empty), then every H1 row of the pair is the OR of the staged rows of N(c): the ranks
// are taken once per (pair, z), not per (pair, c, z in N(c)), and the pair's n output rows are
// written as one contiguous stretch.  A block takes as many consecutive pairs per round as
// give each of its threads a unit of work (one pair for 256 threads at n = 128, four for the
// batch kernel's 1024); rows wider than the staging area go one pair at a time in word chunks.
__host__ __device__ inline int pair_chunk_words(int n, int S, int rwp) {
    const int budget = kPairStageWords / n;
    const int w = S * rwp;
    if (w <= budget) return w;
    return (rwp & 3) == 0 ? (budget & ~3) : budget;
}
__host__ __device__ inline int pair_smem_words(int n) { return rank_table_words(3, n) + kPairStageWords; }

__device__ CR_BODY_INLINE void pair_h1_body(const V1Dev& d, int nx, unsigned wk, unsigned nwk) {
    extern __shared__ uint32_t sm[];
    __shared__ uint32_t s_xy[32];
    constexpr int K = 3;
    const int n = d.g.n, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (!d.h1 || mi.hi < mi.lo || mi.seed || frontier_sparse(d, mi)) return;
    const int s_used = min(mi.hi - mi.base + 1, S);
    const int nwords = s_used * rwp;
    const int np1 = n + 1;
    uint32_t* sB = sm;
    uint32_t* stage = sm + rank_table_words(K, n);
    for (int i = threadIdx.x; i < K * np1; i += blockDim.x) sB[i] = CR_LDG(&d.binom[i]);
    const uint32_t* CR_RESTRICT fin = d.front + (size_t)nx * d.C * S * rwp;
    const uint8_t* CR_RESTRICT fflag_in = d.fflag + (size_t)nx * d.C;
    const uint32_t* CR_RESTRICT rp = cop_rows(d.g);
    const uint16_t* CR_RESTRICT adj = cop_cols(d.g);
    const bool vec4 = (rwp & 3) == 0;
    const int U = vec4 ? 4 : 1;
    const int wc = pair_chunk_words(n, S, rwp);
    const size_t rstride = (size_t)S * rwp;
    const uint32_t P = (uint32_t)(n * (n + 1) / 2);
    // pairs per round: enough units for every thread of the block when a row is staged whole
    int PR = 1;
    if (wc >= nwords) {
        PR = (int)blockDim.x / (n * (nwords / U));
        PR = max(1, min(PR, min(32, kPairStageWords / (n * wc))));
    }
    unsigned err = 0;
    for (uint32_t q0 = wk * PR; q0 < P; q0 += nwk * PR) {
        const int np = (int)min((uint32_t)PR, P - q0);
        if ((int)threadIdx.x < np) {
            int x, y;
            pair_of(q0 + threadIdx.x, n, x, y);
            s_xy[threadIdx.x] = (uint32_t)x | ((uint32_t)y << 16);
        }
        __syncthreads();
        uint32_t* out = d.h1 + (size_t)q0 * n * rstride;
        for (int w0 = 0; w0 < nwords; w0 += wc) {
            const int upr = min(wc, nwords - w0) / U;   // units (of U words) per row
            const int per = n * upr;                    // units per pair
            for (int i = threadIdx.x; i < np * per; i += blockDim.x) {
                const int j = i / per, rem = i - j * per;
                const int z = rem / upr, u = rem - z * upr;
                const uint32_t xy = s_xy[j];
                const int x = (int)(xy & 0xFFFFu), y = (int)(xy >> 16);
                int cc[K];
                cc[0] = z < x ? z : x;
                cc[1] = z < x ? x : (z < y ? z : y);
                cc[2] = z < y ? y : z;
                uint32_t s = rank_s<K>(cc, sB, np1);
                const bool bad = s >= d.C;
                if (bad) {
                    err |= kErrRank;
                    s = 0;
                }
                const bool live = !bad && CR_LDG(&fflag_in[s]) != 0;
                const uint32_t* src = fin + (size_t)s * rstride + w0 + u * U;
                uint32_t* dst = stage + (j * n + z) * wc + u * U;
                if (vec4) {
                    uint4 v = CR_LDG(reinterpret_cast<const uint4*>(src));
                    if (!live) v = make_uint4(0u, 0u, 0u, 0u);
                    *reinterpret_cast<uint4*>(dst) = v;
                } else {
                    const uint32_t v = CR_LDG(src);
                    dst[0] = live ? v : 0u;
                }
            }
            __syncthreads();
            for (int i = threadIdx.x; i < np * per; i += blockDim.x) {
                const int j = i / per, rem = i - j * per;
                const int c = rem / upr, u = rem - c * upr;
                const uint32_t e1 = CR_LDG(&rp[c + 1]);
                const uint32_t* sj = stage + j * n * wc + u * U;
                uint32_t* o = out + ((size_t)j * n + c) * rstride + w0 + u * U;
                if (vec4) {
                    uint4 a = make_uint4(0u, 0u, 0u, 0u);
                    for (uint32_t e = CR_LDG(&rp[c]); e < e1; ++e) {
                        const uint4 v = *reinterpret_cast<const uint4*>(sj + CR_LDG(&adj[e]) * wc);
                        a.x |= v.x; a.y |= v.y; a.z |= v.z; a.w |= v.w;
                    }
                    *reinterpret_cast<uint4*>(o) = a;
                } else {
                    uint32_t a = 0u;
                    for (uint32_t e = CR_LDG(&rp[c]); e < e1; ++e) a |= sj[CR_LDG(&adj[e]) * wc];
                    o[0] = a;
                }
            }
            __syncthreads();
        }
    }
    err = __reduce_or_sync(FULL_MASK, err);
    if ((threadIdx.x & 31) == 0 && err) atomicOr(d.err, err);
}

// Stage 2: a lane group per configuration, its lanes over the deg^2 pairs (x, y).
template <int NWP, int G>
__device__ CR_BODY_INLINE void sep_pull_body(const V1Dev& d, int col, int nx, unsigned wk, unsigned nwk) {
    extern __shared__ uint32_t sm[];
    constexpr int K = 3;
    constexpr int CPW = 32 / G;
    const int warp = threadIdx.x >> 5;
    const Lanes<G> L(threadIdx.x & 31);
    const int gl = L.glane;
    const int n = d.g.n, rw = d.g.rw, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (!d.h1 || mi.hi < mi.lo || mi.seed || frontier_sparse(d, mi)) return;
    const int base_in = mi.base;
    const int s_used = min(mi.hi - base_in + 1, S);
    const int nwords = s_used * rwp;
    const int out_base = d.meta[col].base;
    const int append = d.meta[col].append;
    uint32_t* wacc = sm + (warp * CPW + L.grp) * (2 * S * rwp);
    uint32_t* wnew = wacc + S * rwp;
    const uint32_t* CR_RESTRICT rp = cop_rows(d.g);
    const uint16_t* CR_RESTRICT adj = cop_cols(d.g);
    const uint32_t* CR_RESTRICT h1 = d.h1;
    const bool vec4 = (rwp & 3) == 0;
    const size_t rstride = (size_t)S * rwp;
    Tally t;
    const size_t step = (size_t)nwk * (blockDim.x >> 5) * CPW;
    for (size_t cb = ((size_t)wk * (blockDim.x >> 5) + warp) * CPW; cb < d.C; cb += step) {
        const uint32_t cid = (uint32_t)(cb + L.grp);
        const bool ok = cid < d.C;
        const uint32_t vm = (ok && gl < rw) ? valid_mask(n, gl) : 0u;
        const uint32_t m = (ok && gl < rw) ? d.marked[((size_t)col * d.C + cid) * rwp + gl] : 0u;
        const bool full = L.all(m == vm);
        const bool need = ok && !full;
        if (!__any_sync(FULL_MASK, need)) continue;
        int lo0 = 0, dg0 = 0, lo1 = 0, dg1 = 0, c3 = 0;
        if (need) {
            const uint16_t* cc = d.configs + (size_t)cid * K;
            const int v0 = cc[0], v1 = cc[1];
            c3 = cc[2];
            lo0 = CR_LDG(&rp[v0]);
            dg0 = CR_LDG(&rp[v0 + 1]) - lo0;
            lo1 = CR_LDG(&rp[v1]);
            dg1 = CR_LDG(&rp[v1 + 1]) - lo1;
        }
        const int T = dg0 * dg1;
        uint32_t acc[NWP];
#pragma unroll
        for (int i = 0; i < NWP; ++i) acc[i] = 0u;
        // odometer over N(c1) x N(c2): this lane starts at pair gl and steps by G
        int i0 = 0, i1 = 0;
        if (T > 0) {
            i0 = gl / dg1;
            i1 = gl - i0 * dg1;
        }
#pragma unroll 2
        for (int tt = gl; tt < T; tt += G) {
            const int xa = CR_LDG(&adj[lo0 + i0]), yb = CR_LDG(&adj[lo1 + i1]);
            const uint32_t q = xa <= yb ? pair_index(xa, yb, n) : pair_index(yb, xa, n);
            const uint32_t* hr = h1 + ((size_t)q * n + c3) * rstride;
            if (vec4) {
#pragma unroll
                for (int w = 0; w < NWP; w += 4) {
                    if (w < nwords) {
                        const uint4 v = CR_LDG(reinterpret_cast<const uint4*>(hr + w));
                        acc[w] |= v.x; acc[w + 1] |= v.y; acc[w + 2] |= v.z; acc[w + 3] |= v.w;
                    }
                }
            } else {
#pragma unroll
                for (int w = 0; w < NWP; ++w)
                    if (w < nwords) acc[w] |= CR_LDG(hr + w);
            }
            i1 += G;
            while (i1 >= dg1 && i0 < dg0) {
                i1 -= dg1;
                ++i0;
            }
        }
        group_or<NWP, G>(acc, gl, wacc, need ? nwords : 0);
        __syncwarp();
        emit_row<G>(d, cid, need, col, m, wacc, wnew, base_in, s_used, out_base, append, L, t);
    }
    t.flush(d, col, L.lane);
}

// Cop turn from the capture seeds (column 1 before pass 1): OR over T(C) of the seed rows
// {r : r in C'} is the union of the cops' neighbourhoods (empty if a cop has no move), so no
// successor is visited.  All seed values are 0: one slot.
template <int K, int G>
__device__ CR_BODY_INLINE void cop_seed_body(const V1Dev& d, int col, int nx, unsigned wk, unsigned nwk) {
    extern __shared__ uint32_t sm[];
    constexpr int CPW = 32 / G;
    const int warp = threadIdx.x >> 5;
    const Lanes<G> L(threadIdx.x & 31);
    const int gl = L.glane;
    const int n = d.g.n, rw = d.g.rw, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (!mi.seed || mi.hi < mi.lo) return;
    const int out_base = d.meta[col].base;
    const int append = d.meta[col].append;
    uint32_t* wacc = sm + (warp * CPW + L.grp) * (2 * S * rwp);
    uint32_t* wnew = wacc + S * rwp;
    const uint32_t* CR_RESTRICT rp = cop_rows(d.g);     // the cops' moves
    Tally t;
    const size_t step = (size_t)nwk * (blockDim.x >> 5) * CPW;
    for (size_t cb = ((size_t)wk * (blockDim.x >> 5) + warp) * CPW; cb < d.C; cb += step) {
        const uint32_t cid = (uint32_t)(cb + L.grp);
        const bool ok = cid < d.C;
        const uint32_t vm = (ok && gl < rw) ? valid_mask(n, gl) : 0u;
        const uint32_t m = (ok && gl < rw) ? d.marked[((size_t)col * d.C + cid) * rwp + gl] : 0u;
        const bool full = L.all(m == vm);
        const bool need = ok && !full;
        if (!__any_sync(FULL_MASK, need)) continue;
        if (need && gl < rwp) {
            const uint16_t* cc = d.configs + (size_t)cid * K;
            uint32_t x = 0;
            bool moves = true;
#pragma unroll
            for (int i = 0; i < K; ++i) {
                const int v = cc[i];
                moves &= CR_LDG(&rp[v + 1]) > CR_LDG(&rp[v]);
                x |= CR_LDG(&d.g.nbr[(size_t)v * rwp + gl]);
            }
            wacc[gl] = moves ? x : 0u;
        }
        __syncwarp();
        emit_row<G>(d, cid, need, col, m, wacc, wnew, mi.base, 1, out_base, append, L, t);
    }
    t.flush(d, col, L.lane);
}

// Sparse cop turn, scatter: every row of column nx's frontier list is ORed into the candidate
// rows of its predecessors (the product of the cops' in-neighbour lists).  A warp takes one list
// entry at a time (entries go to the warps round robin, so the work per warp is one entry's
// predecessor count, whatever the rows' order) and its lanes take the predecessor tuples.  The
// first scatter into a candidate row lists it: a test-and-set in the candidate bitmap, and one
// list atomic per warp and round.  Each entry's flag is cleared as it is taken.
template <int K>
__device__ CR_BODY_INLINE void cop_push_body(const V1Dev& d, int col, int nx, unsigned wk, unsigned nwk) {
    extern __shared__ uint32_t sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = d.g.n, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (mi.seed || !frontier_sparse(d, mi)) return;           // a dense form takes this frontier
    if (wk == 0 && threadIdx.x == 0) d.meta[nx].clean = 1;   // every listed flag is cleared below
    if (mi.hi < mi.lo) return;
    const int s_used = min(mi.hi - mi.base + 1, S);
    const int nwords = s_used * rwp;
    uint32_t* wrow = sm + warp * (S * rwp);
    const uint32_t* CR_RESTRICT fin = d.front + (size_t)nx * d.C * S * rwp;
    uint8_t* fflag_in = d.fflag + (size_t)nx * d.C;
    const uint32_t* CR_RESTRICT rrp = d.g.rrow_ptr;
    const uint16_t* CR_RESTRICT radj = d.g.rcol;
    const int np1 = n + 1;
    const RowList rl(d, nx, mi);
    unsigned err = 0;
    const uint32_t nwarps = nwk * (blockDim.x >> 5);
    for (uint32_t i = wk * (blockDim.x >> 5) + warp; i < rl.n; i += nwarps) {
        const uint32_t cp = rl.id(i);
        const uint32_t* row = fin + (size_t)cp * S * rwp;
        uint32_t nz = 0;
        for (int e = lane; e < nwords; e += 32) {
            const uint32_t v = row[e];
            wrow[e] = v;
            nz |= v;
        }
        if (lane == 0) fflag_in[cp] = 0;
        const bool any = __any_sync(FULL_MASK, nz != 0);
        __syncwarp();
        if (any) {
            const uint16_t* cc = d.configs + (size_t)cp * K;
            int lo[K], dg[K];
            int T = 1;
#pragma unroll
            for (int q = 0; q < K; ++q) {
                const int v = cc[q];
                lo[q] = CR_LDG(&rrp[v]);
                dg[q] = CR_LDG(&rrp[v + 1]) - lo[q];
                T *= dg[q];
            }
            for (int t0 = 0; t0 < T; t0 += 32) {   // T is the warp's: every lane runs each round
                const int tt = t0 + lane;
                bool fresh = false;
                uint32_t pc = 0;
                if (tt < T) {
                    int c[K];
                    int rem = tt;
#pragma unroll
                    for (int q = K - 1; q >= 0; --q) {
                        const int qq = rem / dg[q];
                        c[q] = CR_LDG(&radj[lo[q] + rem - qq * dg[q]]);
                        rem = qq;
                    }
                    sort_small<K>(c);
                    pc = rank_g<K>(c, d.binom, np1);
                    if (pc >= d.C) {
                        err |= kErrRank;
                    } else {
                        uint32_t* crow = d.cand + (size_t)pc * S * rwp;
                        for (int e = 0; e < nwords; ++e)
                            if (wrow[e]) atomicOr(&crow[e], wrow[e]);
                        const uint32_t bit = 1u << (pc & 31);
                        fresh = !(atomicOr(&d.cbits[pc >> 5], bit) & bit);
                    }
                }
                const unsigned b = __ballot_sync(FULL_MASK, fresh);
                if (b) {
                    const int leader = __ffs(b) - 1;
                    unsigned at = 0;
                    if (lane == leader) at = atomicAdd(&d.sync[1], (unsigned)__popc(b));
                    at = __shfl_sync(FULL_MASK, at, leader);
                    if (fresh) d.clist[at + __popc(b & ((1u << lane) - 1u))] = pc;
                }
            }
        }
        __syncwarp();
    }
    err = __reduce_or_sync(FULL_MASK, err);
    if (lane == 0 && err) atomicOr(d.err, err);
}

// Sparse cop turn, mark: the listed candidate rows, CPW per warp at a time.  The rows and their
// bitmap bits are cleared for the next push by the following prep (write-only stores there;
// zeroing each row right after reading it here cost six times the reads).
template <int G>
__device__ CR_BODY_INLINE void cop_apply_body(const V1Dev& d, int col, int nx, unsigned wk, unsigned nwk) {
    extern __shared__ uint32_t sm[];
    constexpr int CPW = 32 / G;
    const int warp = threadIdx.x >> 5;
    const Lanes<G> L(threadIdx.x & 31);
    const int gl = L.glane;
    const int rw = d.g.rw, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (mi.hi < mi.lo || mi.seed || !frontier_sparse(d, mi)) return;
    const int base_in = mi.base;
    const int s_used = min(mi.hi - base_in + 1, S);
    const int out_base = d.meta[col].base;
    const int append = d.meta[col].append;
    uint32_t* wacc = sm + (warp * CPW + L.grp) * (2 * S * rwp);
    uint32_t* wnew = wacc + S * rwp;
    const uint32_t items = d.sync[1];
    Tally t;
    const uint32_t step = nwk * (blockDim.x >> 5) * CPW;
    for (uint32_t b0 = (wk * (blockDim.x >> 5) + warp) * CPW; b0 < items; b0 += step) {
        const uint32_t li = b0 + L.grp;
        const bool valid = li < items;
        const uint32_t cid = valid ? d.clist[li] : 0u;
        uint32_t m = 0;
        if (valid) {
            const uint32_t* crow = d.cand + (size_t)cid * S * rwp;
            for (int e = gl; e < S * rwp; e += G) wacc[e] = crow[e];
            if (gl < rw) m = d.marked[((size_t)col * d.C + cid) * rwp + gl];
        }
        __syncwarp();
        emit_row<G>(d, cid, valid, col, m, wacc, wnew, base_in, s_used, out_base, append, L, t);
    }
    t.flush(d, col, L.lane);
}

// Deferred robber turn (odd column below the last): (C, r, c) = 1 + (C, r, c+1), row-local,
// over column nx's row list (each entry's flag cleared as it is taken).
template <int G>
__device__ CR_BODY_INLINE void direct_body(const V1Dev& d, int col, int nx, unsigned wk, unsigned nwk) {
    extern __shared__ uint32_t sm[];
    constexpr int CPW = 32 / G;
    const int warp = threadIdx.x >> 5;
    const Lanes<G> L(threadIdx.x & 31);
    const int gl = L.glane;
    const int rw = d.g.rw, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (wk == 0 && threadIdx.x == 0) d.meta[nx].clean = 1;   // every listed flag is cleared below
    if (mi.hi < mi.lo) return;
    const int base_in = mi.base;
    const int s_used = min(mi.hi - base_in + 1, S);
    const int out_base = d.meta[col].base;
    const int append = d.meta[col].append;
    uint32_t* wacc = sm + (warp * CPW + L.grp) * (2 * S * rwp);
    uint32_t* wnew = wacc + S * rwp;
    uint8_t* fflag_in = d.fflag + (size_t)nx * d.C;
    const RowList rl(d, nx, mi);
    Tally t;
    const uint32_t step = nwk * (blockDim.x >> 5) * CPW;
    for (uint32_t b0 = (wk * (blockDim.x >> 5) + warp) * CPW; b0 < rl.n; b0 += step) {
        const uint32_t li = b0 + L.grp;
        const bool valid = li < rl.n;
        const uint32_t cid = valid ? rl.id(li) : 0u;
        uint32_t m = 0;
        if (valid) {
            const uint32_t* row = d.front + ((size_t)nx * d.C + cid) * S * rwp;
            for (int e = gl; e < S * rwp; e += G) wacc[e] = e < s_used * rwp ? row[e] : 0u;
            if (gl == 0) fflag_in[cid] = 0;
            if (gl < rw) m = d.marked[((size_t)col * d.C + cid) * rwp + gl];
        }
        __syncwarp();
        emit_row<G>(d, cid, valid, col, m, wacc, wnew, base_in, s_used, out_base, append, L, t);
    }
    t.flush(d, col, L.lane);
}

// Last column (robber move cashed out over the exact-p-hop cloud) from column 0.
// A lane group per configuration whose column-0 row changed; the work is row-local.  Three
// forms per row, whichever touches the fewest vertices:
//   touch (few column-0 marks): only an r whose hop(r) meets the marked row can be complete
//          (or an r with empty hop(r)); those are the OR of the transposed hop rows of the
//          marked vertices, and only they are tested;
//   block (few column-0 vertices unmarked): the open r that some unmarked u blocks are the OR
//          of the transposed hop rows of those u; every other open r is complete;
//   test  (few open r): every open r tests hop(r) within column 0's marked row.
// Only the states found complete read column 0's table bytes (for the max).
//
// Fresh form, used when every older column-0 mark has a value no larger than the smallest value
// of this pass's column-0 marks (old_hi <= lo; true on every pass measured, and the test is
// exact either way): an open r that is complete now but was not complete before has a fresh
// mark in hop(r), and the max over hop(r) is the largest fresh value there.  The fresh marks
// are column 0's frontier rows, one per value slot, so per slot from the top the OR of the
// transposed hop rows of that slot's fresh marks gives the robbers whose max is that slot's
// value; those robbers are then tested for completeness (block or test form) and no table byte
// is read.  An open r complete without a fresh mark in hop(r) was complete at the pass that
// made its last mark and stayed unmarked then, so its value is at least 127 and it stays
// unmarked; an r with empty hop(r) has value 1.
template <bool P1, int G>
__device__ CR_BODY_INLINE void and_body(const V1Dev& d, int col, unsigned wk, unsigned nwk) {
    extern __shared__ uint32_t sm[];
    constexpr int CPW = 32 / G;
    const int warp = threadIdx.x >> 5;
    const Lanes<G> L(threadIdx.x & 31);
    const int gl = L.glane;
    const int n = d.g.n, rw = d.g.rw, rwp = d.g.rwp, S = d.S, cols = d.cols;
    const ColMeta mi = d.meta[0];
    if (wk == 0 && threadIdx.x == 0) d.meta[0].clean = 1;   // every listed flag is cleared below
    if (mi.hi < mi.lo) return;
    const int out_base = d.meta[col].base;
    const int per_grp = and_group_words(S, rwp);
    uint32_t* wm0 = sm + (warp * CPW + L.grp) * per_grp;
    uint32_t* wmc = wm0 + rwp;
    uint32_t* wtouch = wmc + rwp;
    uint32_t* wnew = wtouch + rwp;
    uint8_t* fflag0 = d.fflag;
    // the row tests' graph arrays (transposed hop rows, CSR), staged in shared memory when
    // the launch left room for them; read through generic pointers either way
    const uint32_t* rp = d.g.row_ptr;
    const uint16_t* adj = d.g.col;
    const uint32_t* rhop = d.g.rhop;
    const int nnz = (int)rp[n];
    const RowList rl(d, 0, mi);
    const uint32_t step = nwk * (blockDim.x >> 5) * CPW;
    if (wk * (blockDim.x >> 5) * CPW >= rl.n) return;   // no row for this block
    // staging pays off only when each lane group takes a few rows
    if (d.and_stage_words && rl.n >= 2u * step) {
        const uint32_t need = (uint32_t)(n * rwp + n + 1) + (uint32_t)(nnz + 1) / 2;
        if (need <= d.and_stage_words) {
            uint32_t* st = sm + (blockDim.x >> 5) * CPW * per_grp;
            uint32_t* srp = st + n * rwp;
            uint16_t* sadj = reinterpret_cast<uint16_t*>(srp + n + 1);
            for (int i = threadIdx.x; i < n * rwp; i += blockDim.x) st[i] = rhop[i];
            for (int i = threadIdx.x; i <= n; i += blockDim.x) srp[i] = rp[i];
            for (int i = threadIdx.x; i < nnz; i += blockDim.x) sadj[i] = adj[i];
            __syncthreads();
            rhop = st;
            rp = srp;
            adj = sadj;
        }
    }
    const int avg_deg = max(1, (nnz + n - 1) / n);
    const int slo = mi.lo - mi.base, shi = mi.hi - mi.base;
    const bool fresh = d.fresh_last && mi.old_hi <= mi.lo && slo >= 0 && shi < S;
    Tally t;
    for (uint32_t b0 = (wk * (blockDim.x >> 5) + warp) * CPW; b0 < rl.n; b0 += step) {
        {
            const uint32_t li = b0 + L.grp;
            const bool valid = li < rl.n;
            const uint32_t cid = valid ? rl.id(li) : 0u;
            if (valid && gl == 0) fflag0[cid] = 0;
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
            }
            if (need)
                for (int e = gl; e < S * rwp; e += G) wnew[e] = 0u;
            const int marked0 = L.sum(__popc(m0));
            constexpr bool kBlockRows = G <= 4;
            __syncwarp();
            if (fresh) {
                const uint32_t open = (need && gl < rw) ? (~mc & vm) : 0u;
                uint32_t done = 0u;   // open robbers whose hop(r) meets a fresh mark of a slot seen
                const uint32_t* frow0 = d.front + (size_t)cid * S * rwp;
                for (int s = shi; s >= slo; --s) {
                    const uint32_t fs = (need && gl < rw) ? frow0[s * rwp + gl] : 0u;
                    if (!__any_sync(FULL_MASK, fs != 0u)) continue;
                    uint32_t acc[G];
#pragma unroll
                    for (int i = 0; i < G; ++i) acc[i] = 0u;
                    uint32_t mb = fs;
                    while (mb) {
                        const uint32_t* row = rhop + (size_t)(gl * 32 + __ffs(mb) - 1) * rwp;
                        mb &= mb - 1;
#pragma unroll
                        for (int w = 0; w < G; ++w)
                            if (w < rwp) acc[w] |= row[w];
                    }
                    group_or<G, G>(acc, gl, wtouch, L.any(fs != 0u) ? rwp : 0);
                    __syncwarp();
                    if (L.any(fs != 0u) && gl < rw) {
                        const uint32_t tw = wtouch[gl] & open & ~done;
                        done |= tw;
                        const int v = mi.base + s + 1;
                        if (tw && v < kMaxRound) {
                            const int so = v - out_base;
                            if (so < 0 || so >= S) t.err |= kErrSlot;
                            else wnew[so * rwp + gl] = tw;
                        }
                    }
                    __syncwarp();
                }
                // completeness of the touched robbers: the blocked set (OR of the transposed hop
                // rows of the unmarked column-0 vertices) or a test per robber, whichever is cheaper
                const int ncand = L.sum(__popc(done));
                const bool block_form = (n - marked0) * rwp < ncand * (P1 ? avg_deg : rw);
                const bool do_block = need && ncand > 0 && block_form;
                uint32_t comp = done;
                if (kBlockRows) {
                    if (__any_sync(FULL_MASK, do_block)) {
                        uint32_t acc[G];
#pragma unroll
                        for (int i = 0; i < G; ++i) acc[i] = 0u;
                        uint32_t mb = (do_block && gl < rw) ? (~m0 & vm) : 0u;
                        while (mb) {
                            const uint32_t* row = rhop + (size_t)(gl * 32 + __ffs(mb) - 1) * rwp;
                            mb &= mb - 1;
#pragma unroll
                            for (int w = 0; w < G; ++w)
                                if (w < rwp) acc[w] |= row[w];
                        }
                        group_or<G, G>(acc, gl, wtouch, do_block ? rwp : 0);
                        __syncwarp();
                        if (do_block && gl < rw) comp &= ~wtouch[gl];
                    }
                } else if (do_block && gl < rw) {
                    uint32_t blocked = 0;
                    for (int w2 = 0; w2 < rw; ++w2) {
                        uint32_t ub = ~wm0[w2] & valid_mask(n, w2);
                        while (ub) {
                            const int u = w2 * 32 + __ffs(ub) - 1;
                            ub &= ub - 1;
                            blocked |= rhop[(size_t)u * rwp + gl];
                        }
                    }
                    comp &= ~blocked;
                }
                if (need && !block_form && gl < rw) {
                    uint32_t c = done;
                    comp = 0u;
                    while (c) {
                        const int r = gl * 32 + __ffs(c) - 1;
                        c &= c - 1;
                        bool all = true;
                        if (P1) {
                            const uint32_t e1 = rp[r + 1];
                            for (uint32_t e = rp[r]; e < e1 && all; ++e) {
                                const int v = adj[e];
                                all = (wm0[v >> 5] >> (v & 31)) & 1u;
                            }
                        } else {
                            const uint32_t* h = d.hop + (size_t)r * rwp;
                            for (int w = 0; w < rw && all; ++w) all = (CR_LDG(&h[w]) & ~wm0[w]) == 0u;
                        }
                        if (all) comp |= 1u << (r & 31);
                    }
                }
                if (need && gl < rw) {
                    for (int so = 0; so < S; ++so) wnew[so * rwp + gl] &= comp;
                    // an open r with empty hop(r): value 1
                    const uint32_t iso = open & CR_LDG(&d.g.isolated[gl]);
                    if (iso) {
                        const int so = 1 - out_base;
                        if (so < 0 || so >= S) t.err |= kErrSlot;
                        else wnew[so * rwp + gl] |= iso;
                    }
                    uint8_t* tcol = d.table + ((size_t)cid * n + gl * 32) * cols + col;
                    for (int so = 0; so < S; ++so) {
                        uint32_t b = wnew[so * rwp + gl];
                        if (!b) continue;
                        const int v = out_base + so;
                        t.lo = min(t.lo, v);
                        t.hi = max(t.hi, v);
                        const uint8_t val = (uint8_t)(1 | (v << 1));
                        while (b) {
                            tcol[(size_t)(__ffs(b) - 1) * cols] = val;
                            b &= b - 1;
                        }
                    }
                }
            } else {
                const int open = L.sum(__popc(~mc & vm));
                const int c_test = open * (P1 ? avg_deg : rw);
                const int c_block = (n - marked0) * rwp;
                const int c_touch = marked0 * rwp + (P1 ? marked0 * avg_deg : open);
                const bool touch_form = c_touch < c_test && c_touch <= c_block;
                const bool block_form = !touch_form && c_block < c_test;
                // block form with groups of up to 4 lanes (n <= 128): each lane walks the unmarked
                // vertices of its own word and ORs whole rows, like the touch form; wider groups
                // keep one pass per lane over the whole list (clustered unmarked vertices would
                // leave a few lanes with all the rows)
                const bool rows_form = touch_form || (kBlockRows && block_form);
                if (__any_sync(FULL_MASK, rows_form && need)) {
                    // each lane ORs the transposed hop rows of the marked (touch form) or unmarked
                    // (block form) vertices of its own word; the group reduces the rows by halving
                    // into wtouch: the touched, or the blocked, robbers
                    uint32_t acc[G];
    #pragma unroll
                    for (int i = 0; i < G; ++i) acc[i] = 0u;
                    if (rows_form && need && gl < rw) {
                        uint32_t mb = touch_form ? m0 : (~m0 & vm);
                        while (mb) {
                            const int v = gl * 32 + __ffs(mb) - 1;
                            mb &= mb - 1;
                            const uint32_t* row = rhop + (size_t)v * rwp;
    #pragma unroll
                            for (int w = 0; w < G; ++w)
                                if (w < rwp) acc[w] |= row[w];
                        }
                    }
                    group_or<G, G>(acc, gl, wtouch, (rows_form && need) ? rwp : 0);
                }
                __syncwarp();
                if (need && gl < rw) {
                    const uint8_t* trow = d.table + (size_t)cid * n * cols;
                    // candidates: touched and open (count form), open and not blocked (block form,
                    // all of them complete), or every open state (test form)
                    uint32_t cand = ~mc & vm;
                    if (touch_form) cand &= wtouch[gl] | CR_LDG(&d.g.isolated[gl]);
                    if (block_form) {
                        if (kBlockRows) {
                            cand &= ~wtouch[gl];
                        } else {
                            uint32_t blocked = 0;
                            for (int w2 = 0; w2 < rw; ++w2) {
                                uint32_t ub = ~wm0[w2] & valid_mask(n, w2);
                                while (ub) {
                                    const int u = w2 * 32 + __ffs(ub) - 1;
                                    ub &= ub - 1;
                                    blocked |= rhop[(size_t)u * rwp + gl];
                                }
                            }
                            cand &= ~blocked;
                        }
                    }
                    while (cand) {
                        const int r = gl * 32 + __ffs(cand) - 1;
                        cand &= cand - 1;
                        const uint32_t e0 = rp[r], e1 = rp[r + 1];
                        bool all;
                        int mx = 0;
                        if (P1) {
                            if (block_form) {
                                all = true;
                            } else {
                                all = true;
                                for (uint32_t e = e0; e < e1 && all; ++e) {
                                    const int v = adj[e];
                                    all = (wm0[v >> 5] >> (v & 31)) & 1u;
                                }
                            }
                            if (all)
                                for (uint32_t e = e0; e < e1; ++e)
                                    mx = max(mx, (int)(trow[(size_t)adj[e] * cols] >> 1));
                        } else {
                            const uint32_t* h = d.hop + (size_t)r * rwp;
                            all = true;
                            if (!block_form)
                                for (int w = 0; w < rw && all; ++w) all = (CR_LDG(&h[w]) & ~wm0[w]) == 0u;
                            if (all) {
                                for (int w = 0; w < rw; ++w) {
                                    uint32_t b = CR_LDG(&h[w]);
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
            }
            __syncwarp();
            uint32_t nb = 0;
            if (need && gl < rw)
                for (int s = 0; s < S; ++s) nb |= wnew[s * rwp + gl];
            const bool newrow = L.any(nb != 0);
            if (newrow) {
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
            t.append(d, col, newrow && gl == 0, cid, L.lane);
            __syncwarp();
        }
    }
    t.flush(d, col, L.lane);
}

// findFinalResult (k_cops_visibility.cpp:301-331): over the configurations whose column-0 row
// is all marked, the smallest (worst capture round, config id) key.  A warp takes 32
// configurations at a time, each lane testing its own row's marks; the warp then reads each
// full row (two columns: one 16-byte load per lane covers 8 robbers, 256 per step) and keeps a
// per-lane running minimum, reduced once per warp into one atomic.
__device__ CR_BODY_INLINE void verdict_body(const uint8_t* table, const uint32_t* m0, uint32_t C,
                                             int n, int rw, int rwp, int cols,
                                             unsigned long long* best, unsigned wk, unsigned nwk) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t stride = (size_t)nwk * blockDim.x;
    const bool vec = cols == 2 && (n & 7) == 0 && ((uintptr_t)table & 15u) == 0;
    unsigned long long mine = ~0ull;
    for (size_t base = (size_t)wk * blockDim.x + warp * 32; base < C; base += stride) {
        const size_t cid = base + lane;
        bool full = cid < C;
        for (int w = 0; w < rw && full; ++w) full = m0[cid * rwp + w] == valid_mask(n, w);
        unsigned act = __ballot_sync(FULL_MASK, full);
        while (act) {
            const size_t c = base + __ffs(act) - 1;
            act &= act - 1;
            const uint8_t* row = table + c * n * cols;
            uint32_t wc = 0;
            if (vec) {
                for (int r0 = lane * 8; r0 < n; r0 += 256) {
                    const uint4 v = *reinterpret_cast<const uint4*>(row + r0 * 2);
                    // column-0 bytes are the even bytes; round = byte >> 1
                    const uint32_t e0 = __byte_perm(v.x, v.y, 0x6420), e1 = __byte_perm(v.z, v.w, 0x6420);
                    const uint32_t m = __vmaxu4(e0 >> 1 & 0x7F7F7F7Fu, e1 >> 1 & 0x7F7F7F7Fu);
                    wc = max(wc, max(max(m & 0xFFu, (m >> 8) & 0xFFu), max((m >> 16) & 0xFFu, m >> 24)));
                }
            } else {
                for (int r = lane; r < n; r += 32) wc = max(wc, (uint32_t)(row[(size_t)r * cols] >> 1));
            }
            wc = __reduce_max_sync(FULL_MASK, wc);
            const unsigned long long key = ((unsigned long long)wc << 32) | c;
            mine = key < mine ? key : mine;
        }
    }
    // every lane holds the same running minimum (the keys are warp-uniform)
    if (lane == 0 && mine != ~0ull) atomicMin(best, mine);
}

}  // namespace CR_BODY_NS
}  // namespace crgpu
