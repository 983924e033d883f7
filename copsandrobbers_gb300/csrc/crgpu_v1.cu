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
// The cop turn runs in one of these forms, chosen on the device from the frontier's row count:
//   seed          the capture seeds of column 1 before pass 1, in closed form: the OR of the
//                 seed rows over T(C) is the union of the cops' neighbourhoods;
//   pull (dense)  every configuration ORs the frontier rows of its successors (k_cop_pull), or
//                 for k = 3 in separable form through pair rows (pair_h1 + sep_pull);
//   push (sparse) every row of the frontier's list is ORed into the candidate rows of its
//                 predecessors with atomics, then only those rows are marked (push + apply).
// k_cop_a and k_cop_b carry the seed, push, apply and separable bodies (each body returns at
// once unless its form applies), so a cop turn is two launches for k = 3 and three otherwise.
#include "crgpu_internal.cuh"

#include <algorithm>

#define CR_BODY_NS grid
#define CR_LDG(p) __ldg(p)
#define CR_RESTRICT __restrict__
#define CR_BODY_INLINE __forceinline__
#include "crgpu_v1_body.cuh"

namespace crgpu {

using namespace grid;

__device__ void list_compact_body(const V1Dev& d, int col);

__global__ void k_prep(V1Dev d, int col, int nx) { prep_body(d, col, nx, blockIdx.x, gridDim.x); }
__global__ void k_init(V1Dev d, int K) { init_body(d, K, blockIdx.x, gridDim.x); }
// The first pass in two instances: rows of one 256-robber block split into whole lane pieces
// (the run form; at most 85 registers, 3 blocks of 256 per SM, which measured faster than 64
// registers at 4 blocks and than 2 blocks), and every other row shape (64 registers).
template <int K, int W, bool SINGLE>
__global__ void __launch_bounds__(256, SINGLE ? 3 : 4) k_init_pass1(V1Dev d) {
    if (SINGLE) {
        if (d.g.n == 256) init_pass1_single<K, W, true>(d, blockIdx.x, gridDim.x);
        else init_pass1_single<K, W, false>(d, blockIdx.x, gridDim.x);
    } else {
        init_pass1_body<K, W>(d, blockIdx.x, gridDim.x);
    }
}

template <int K, int NWP, int G>
__global__ void __launch_bounds__(256) k_cop_pull(V1Dev d, int col, int nx) {
    cop_pull_body<K, NWP, G>(d, col, nx, blockIdx.x, gridDim.x);
}
// The other cop-turn forms share two launches, each body returning at once unless its form
// applies (the form is chosen on the device from the input frontier):
//   k_cop_a  the capture-seed form, the push scatter, or (k = 3) the separable turn's pair rows;
//   k_cop_b  the separable turn's configurations (k = 3) or the push form's marking.
// The tuple-gathering pull (k != 3, or no pair rows) keeps its own launch: it wants up to 127
// registers, the bodies here at most 64 (80 with 32-word rows), being latency-bound.
template <int K, int NWP, int G>
__global__ void __launch_bounds__(256, NWP >= 32 ? 3 : 4) k_cop_a(V1Dev d, int col, int nx) {
    cop_seed_body<K, G>(d, col, nx, blockIdx.x, gridDim.x);
    cop_push_body<K>(d, col, nx, blockIdx.x, gridDim.x);
    if constexpr (K == 3) pair_h1_body(d, nx, blockIdx.x, gridDim.x);
}
template <int K, int NWP, int G>
__global__ void __launch_bounds__(256, NWP >= 32 ? 3 : 4) k_cop_b(V1Dev d, int col, int nx) {
    if constexpr (K == 3) sep_pull_body<NWP, G>(d, col, nx, blockIdx.x, gridDim.x);
    cop_apply_body<G>(d, col, nx, blockIdx.x, gridDim.x);
}
// k_cop_b inside the device-side pass loop of a p = 1 solve, followed by the last column's prep
// (column nx = 1): the flags a dense turn left in column 1 (no body of this launch reads them),
// and in the last block the column's state reset.  The candidate rows wait for the last column.
template <int K, int NWP, int G>
__global__ void __launch_bounds__(256, NWP >= 32 ? 3 : 4) k_cop_b_end(V1Dev d, int col, int nx) {
    if constexpr (K == 3) sep_pull_body<NWP, G>(d, col, nx, blockIdx.x, gridDim.x);
    cop_apply_body<G>(d, col, nx, blockIdx.x, gridDim.x);
    prep_clear_flags(d, nx, blockIdx.x, gridDim.x);
    __syncthreads();
    if (threadIdx.x == 0 && grid_last_block(d, gridDim.x)) prep_reset(d, nx, col);
}
template <int G>
__global__ void __launch_bounds__(256) k_direct(V1Dev d, int col, int nx) {
    direct_body<G>(d, col, nx, blockIdx.x, gridDim.x);
}
// at most 64 registers: the grid runs 4 blocks of 256 per SM (more registers cost occupancy
// that this latency-bound body needs more)
template <bool P1, int G>
__global__ void __launch_bounds__(256, 4) k_and(V1Dev d, int col) {
    and_body<P1, G>(d, col, blockIdx.x, gridDim.x);
}
// The last column inside the device-side pass loop, with the loop's bookkeeping in its last
// block: the pass's count joins the history, the loop goes on while the pass found something
// (no error bit, history not full), and column 0's prep for the next pass runs (this column
// cleared every flag of column 0's list, so that prep is a reset of the column's state).
template <bool P1, int G>
__global__ void __launch_bounds__(256, 4) k_and_end(V1Dev d, int col, LoopCtl c) {
    if (c.fused_prep1) prep_clear_cand(d, blockIdx.x, gridDim.x);   // this column's prep, the rest
    and_body<P1, G>(d, col, blockIdx.x, gridDim.x);
    __syncthreads();
    if (threadIdx.x == 0 && grid_last_block(d, gridDim.x)) {
        const int i = *c.idx;
        const unsigned long long f = *d.pass_new;
        c.hist[i] = f;
        *c.idx = i + 1;
        cudaGraphSetConditional(c.loop, (f != 0ull && *d.err == 0u && i + 1 < c.cap) ? 1u : 0u);
        prep_reset(d, 0, 1);
    }
}

// Entry of the device-side pass loop: column 0's prep for the first pass of the loop; its last
// block records a first pass run just before the loop (*idx = 1, set by the host) as the
// history's first entry and starts the loop if the last pass found something and no error bit
// is set.
__global__ void __launch_bounds__(256) k_loop_enter(V1Dev d, LoopCtl c) {
    // column 1's row list after a fused first pass (every block reads the marker before the
    // last block clears it)
    if (d.meta[1].compact) list_compact_body(d, 1);
    prep_clear(d, 0, blockIdx.x, gridDim.x);
    __syncthreads();
    if (threadIdx.x == 0 && grid_last_block(d, gridDim.x)) {
        d.meta[1].compact = 0;
        const unsigned long long f = *d.pass_new;
        if (*c.idx == 1) c.hist[0] = f;
        cudaGraphSetConditional(c.loop, (f != 0ull && *d.err == 0u) ? 1u : 0u);
        prep_reset(d, 0, 1);
    }
}

__global__ void k_verdict(const uint8_t* __restrict__ table, const uint32_t* __restrict__ m0,
                          uint32_t C, int n, int rw, int rwp, int cols, unsigned long long* best) {
    verdict_body(table, m0, C, n, rw, rwp, cols, best, blockIdx.x, gridDim.x);
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
    (void)n;
    return (size_t)8 * (32 / group_lanes(rwp)) * and_group_words(S, rwp) * sizeof(uint32_t);
}

static int pull_words(int S, int rwp) {
    int w = S * rwp, p = 2;
    while (p < w) p <<= 1;
    return p;
}

bool pull_supported(int S, int rwp) { return pull_words(S, rwp) <= 32 && group_lanes(rwp) <= 32; }

template <int K, int NWP, int G>
static void launch_cop_ng(const V1Dev& d, int col, int nx, int grid, cudaStream_t st, bool end) {
    const size_t sm = cop_smem_bytes(d.S, d.g.rwp);
    const size_t smr = sm + (size_t)rank_table_words(K, d.g.n) * 4;
    const size_t sma = K == 3 ? std::max(smr, (size_t)pair_smem_words(d.g.n) * 4) : smr;
    k_cop_a<K, NWP, G><<<grid, 256, sma, st>>>(d, col, nx);
    if (!(K == 3 && d.h1)) k_cop_pull<K, NWP, G><<<grid, 256, smr, st>>>(d, col, nx);
    if (end) k_cop_b_end<K, NWP, G><<<grid, 256, sm, st>>>(d, col, nx);
    else k_cop_b<K, NWP, G><<<grid, 256, sm, st>>>(d, col, nx);
}

// Accumulator words and lanes per configuration, as the pull and the separable turn use them.
template <int K>
static void launch_cop_k(const V1Dev& d, int col, int nx, int grid, cudaStream_t st, bool end) {
    const int G = group_lanes(d.g.rwp);
    switch (pull_words(d.S, d.g.rwp)) {
        case 2: launch_cop_ng<K, 2, 4>(d, col, nx, grid, st, end); break;
        case 4: launch_cop_ng<K, 4, 4>(d, col, nx, grid, st, end); break;
        case 8: launch_cop_ng<K, 8, 4>(d, col, nx, grid, st, end); break;
        case 16:
            if (G == 4) launch_cop_ng<K, 16, 4>(d, col, nx, grid, st, end);
            else launch_cop_ng<K, 16, 8>(d, col, nx, grid, st, end);
            break;
        default:
            if (G == 4) launch_cop_ng<K, 32, 4>(d, col, nx, grid, st, end);
            else if (G == 8) launch_cop_ng<K, 32, 8>(d, col, nx, grid, st, end);
            else launch_cop_ng<K, 32, 16>(d, col, nx, grid, st, end);
            break;
    }
}

template <int G>
static void launch_direct_g(const V1Dev& d, int col, int nx, int grid, cudaStream_t st) {
    k_direct<G><<<grid, 256, cop_smem_bytes(d.S, d.g.rwp), st>>>(d, col, nx);
}

// Cop turn into column col (or, direct = 1, a deferred robber turn): every form that may apply
// is enqueued; each reads the input frontier's row count on the device and only the matching
// form does work.
void launch_cop(const V1Dev& d, int col, int nx, int direct, int grid, cudaStream_t st, bool end) {
    if (direct) {
        switch (group_lanes(d.g.rwp)) {
            case 4: launch_direct_g<4>(d, col, nx, grid, st); break;
            case 8: launch_direct_g<8>(d, col, nx, grid, st); break;
            case 16: launch_direct_g<16>(d, col, nx, grid, st); break;
            default: launch_direct_g<32>(d, col, nx, grid, st); break;
        }
        return;
    }
    switch (d.k) {
        case 1: launch_cop_k<1>(d, col, nx, grid, st, end); break;
        case 2: launch_cop_k<2>(d, col, nx, grid, st, end); break;
        case 3: launch_cop_k<3>(d, col, nx, grid, st, end); break;
        default: launch_cop_k<4>(d, col, nx, grid, st, end); break;
    }
}

int cop_launches(int direct) { return direct ? 1 : 3; }
int cop_launches_k(int direct, int k, bool sep) { return direct ? 1 : (k == 3 && sep ? 2 : 3); }

// Shared-memory words the last-column body stages the graph in: transposed hop rows, row
// pointers and neighbour lists.
size_t and_stage_words(int n, int rwp, int nnz) {
    return (size_t)n * rwp + n + 1 + (size_t)(nnz + 1) / 2;
}

template <bool P1, int G>
static void launch_and_g(const V1Dev& d, int col, int grid, size_t sm, cudaStream_t st, const LoopCtl* loop) {
    if (loop) k_and_end<P1, G><<<grid, 256, sm, st>>>(d, col, *loop);
    else k_and<P1, G><<<grid, 256, sm, st>>>(d, col);
}

template <bool P1>
static void launch_and_p(const V1Dev& d0, int col, int grid, cudaStream_t st, const LoopCtl* loop) {
    V1Dev d = d0;
    size_t sm = and_smem_bytes(d.S, d.g.rwp, d.g.n);
    d.and_stage_words = 0;
    if (d.g.nnz >= 0) {
        const size_t words = and_stage_words(d.g.n, d.g.rwp, d.g.nnz);
        if (sm + words * 4 <= 48 * 1024) {   // within the default dynamic shared-memory limit
            d.and_stage_words = (uint32_t)words;
            sm += words * 4;
        }
    }
    switch (group_lanes(d.g.rwp)) {
        case 4: launch_and_g<P1, 4>(d, col, grid, sm, st, loop); break;
        case 8: launch_and_g<P1, 8>(d, col, grid, sm, st, loop); break;
        case 16: launch_and_g<P1, 16>(d, col, grid, sm, st, loop); break;
        default: launch_and_g<P1, 32>(d, col, grid, sm, st, loop); break;
    }
}

void launch_and(const V1Dev& d, int col, bool p1, int grid, cudaStream_t st, const LoopCtl* loop) {
    if (p1) launch_and_p<true>(d, col, grid, st, loop);
    else launch_and_p<false>(d, col, grid, st, loop);
}

void launch_loop_enter(const V1Dev& d, const LoopCtl& c, int grid, cudaStream_t st) {
    k_loop_enter<<<grid, 256, 0, st>>>(d, c);
}

void launch_prep(const V1Dev& d, int col, int nx, int grid, cudaStream_t st) {
    k_prep<<<grid, 256, 0, st>>>(d, col, nx);
}

void launch_init(const V1Dev& d, int grid, cudaStream_t st) { k_init<<<grid, 256, 0, st>>>(d, d.k); }

template <int W, bool SINGLE>
static void launch_init_pass1_w(const V1Dev& d, int grid, size_t sm, cudaStream_t st) {
    switch (d.k) {
        case 1: k_init_pass1<1, W, SINGLE><<<grid, 256, sm, st>>>(d); break;
        case 2: k_init_pass1<2, W, SINGLE><<<grid, 256, sm, st>>>(d); break;
        case 3: k_init_pass1<3, W, SINGLE><<<grid, 256, sm, st>>>(d); break;
        default: k_init_pass1<4, W, SINGLE><<<grid, 256, sm, st>>>(d); break;
    }
}
template <bool SINGLE>
static void launch_init_pass1_s(const V1Dev& d, int grid, size_t sm, cudaStream_t st) {
    if (d.g.cover_w == 1) launch_init_pass1_w<1, SINGLE>(d, grid, sm, st);
    else if (d.g.cover_w == 2) launch_init_pass1_w<2, SINGLE>(d, grid, sm, st);
    else launch_init_pass1_w<4, SINGLE>(d, grid, sm, st);
}

// Requires d.g.cover (cover_w 1, 2 or 4) and two columns.  Rows of one 256-robber block
// split into whole lane pieces take the run form, which needs its tables in shared memory.
// One wave of resident blocks: each warp sweeps one contiguous range of configurations.
void launch_init_pass1(const V1Dev& d, int num_sms, cudaStream_t st) {
    const bool single = d.g.n <= 256 && (d.g.n & 7) == 0;
    const uint64_t cap = ((uint64_t)d.C + 7) / 8;
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(cap, (uint64_t)num_sms * (single ? 3 : 4)));
    if (single) launch_init_pass1_s<true>(d, grid, (size_t)init_pass1_smem_words(d.g.n, d.g.rwp) * 4, st);
    else launch_init_pass1_s<false>(d, grid, 0, st);
}

// Builds column col's row list from its flag plane (after the first pass): each block takes
// segments of 16 flags per thread, counts the set ones, reserves its segment's room in the list
// with one atomic and writes the ids (the list order is irrelevant to its consumers).
__device__ void list_compact_body(const V1Dev& d, int col) {
    __shared__ unsigned s_warp[8];
    __shared__ unsigned s_at;
    constexpr int kPer = 16;
    const uint8_t* f = d.fflag + (size_t)col * d.C;
    uint32_t* out = d.list + (size_t)col * d.C;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const size_t seg = (size_t)blockDim.x * kPer;
    for (size_t base = (size_t)blockIdx.x * seg; base < d.C; base += (size_t)gridDim.x * seg) {
        unsigned bits = 0;   // bit j: flag base + j * blockDim.x + threadIdx.x is set
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const size_t i = base + (size_t)j * blockDim.x + threadIdx.x;
            if (i < d.C && f[i]) bits |= 1u << j;
        }
        const unsigned mine = __popc(bits);
        unsigned incl = mine;   // inclusive scan over the warp
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o) incl += v;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned tot = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
                const unsigned c = s_warp[w];
                s_warp[w] = tot;
                tot += c;
            }
            s_at = tot ? (unsigned)atomicAdd(&d.meta[col].len, (int)tot) : 0u;
        }
        __syncthreads();
        unsigned at = s_at + s_warp[warp] + incl - mine;
        while (bits) {
            const int j = __ffs(bits) - 1;
            bits &= bits - 1;
            out[at++] = (uint32_t)(base + (size_t)j * blockDim.x + threadIdx.x);
        }
        __syncthreads();
    }
}
__global__ void __launch_bounds__(256) k_list_compact(V1Dev d, int col) { list_compact_body(d, col); }

void launch_list_compact(const V1Dev& d, int col, int num_sms, cudaStream_t st) {
    const uint64_t segs = ((uint64_t)d.C + 256 * 16 - 1) / (256 * 16);
    const int grid = (int)std::max<uint64_t>(1, std::min<uint64_t>(segs, (uint64_t)num_sms * 4));
    k_list_compact<<<grid, 256, 0, st>>>(d, col);
}

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
