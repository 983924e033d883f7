// crgpu_internal.cuh - device data layout and helpers shared by the solver kernels.
//
// State store (one solve):
//   table   uint8  [C][n][cols]      the reference's states section, byte = marked | round << 1,
//                                    0xFE unmarked (solvers/k_cops_visibility.cpp:20-26,
//                                    index (cId * N + r) * columns + col, AuxGraph.h:96-98)
//   marked  uint32 [cols][C][rwp]    bit r of row C: state (C, r, col) is marked
//   front   uint32 [cols][C][S][rwp] marks the column's last producer run made, split by
//                                    value: slot s holds the states of value base + s
//   fflag   uint8  [cols][C]         1 = row C of the column's frontier is non-empty
//   list    uint32 [cols][C]         the ids of those rows, in append order (meta.len of them)
//   configs uint16 [C][k]            sorted cop multisets in lexicographic order (AuxGraph.h:117-177)
// rw = ceil(n / 32) words of robber bits per row; rwp pads rw to 1, 2 or a multiple of 4 so
// that a row starts on a 16-byte boundary and loads as uint4 vectors.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>

namespace crgpu {

constexpr int kMaxRound = 127;      // MAX_ROUND_COUNT, k_cops_visibility.cpp:26
constexpr int kEmptyLo = 1 << 20;   // "no value yet" for frontier ranges
constexpr uint8_t kUnmarked = 0xFE;

// Device-side error bits (ORed into DevState::err).
constexpr unsigned kErrSlot = 1u;    // a value fell outside the frontier's value slots
constexpr unsigned kErrRank = 2u;    // a successor rank fell outside [0, C)
constexpr unsigned kErrBudget = 4u;  // a bounded device loop ran out

// A frontier with fewer non-empty rows than C / kPushRatio is pushed to its predecessors
// (scatter with atomic ORs); a denser one is pulled by every configuration (gather).
constexpr int kPushRatio = 16;

// Range and base of the value slots of one column's frontier.
struct ColMeta {
    int base;    // value of slot 0
    int lo;      // smallest value in the frontier (kEmptyLo when empty)
    int hi;      // largest value in the frontier (-1 when empty)
    int append;  // 1 = the next producer run adds to the frontier instead of replacing it
    int rows;    // configurations whose frontier row is non-empty
    int seed;    // 1 = the frontier is exactly the capture seeds (r on a cop, value 0)
    int len;     // rows in the column's list; -1 = every configuration (the list is implicit)
    int clean;   // 1 = the frontier's consumer has cleared the flags of the listed rows
    // Largest value among the column's marks made before the current frontier's producer run
    // (captures, value 0, are always among them; value-initialised brace lists leave it 0).
    int old_hi;
    // 1 = the list is still to be built from the flags (by the pass loop's entry kernel)
    int compact;
};

// Candidate rows of the push-mode cop turn: a bitmap of C bits marks the configurations that
// received a candidate row; its bytes (rounded up to whole words).
__host__ __device__ inline size_t cand_bits_bytes(uint64_t C) { return (size_t)((C + 31) / 32) * 4; }

struct DevGraph {
    int n;
    int maxdeg;           // largest out-degree
    int rw;               // 32-bit words per robber row
    int rwp;              // padded words per row
    const uint32_t* row_ptr;  // n + 1
    const uint16_t* col;      // out-neighbours, ascending
    const uint32_t* rrow_ptr; // n + 1: in-neighbours (predecessor moves)
    const uint16_t* rcol;
    const uint32_t* nbr;      // [n][rwp]: out-neighbour masks
    const uint32_t* isolated; // [rwp]: vertices without out-neighbours
    const uint32_t* rhop;     // [n][rwp]: bit r of row u set iff u is in hop(r) (transposed hop)
    // Uncovered-slot masks for the first pass's closed form (cover_w bytes per mask, 0 = not
    // built; npad = n rounded up to 8).  Bit j of a mask refers to r's j-th out-neighbour:
    //   cover[c][r]            bit j set iff that neighbour is neither c nor an out-neighbour of c;
    //                          except cover[c][c] = all ones and, for a cop c without a move,
    //                          cover[c][*] = 0 (read only when every cop can move)
    //   cover[n + c][r]        bit j set iff that neighbour is not c
    const uint8_t* cover;
    int cover_w;
    int npad;
    int nnz = -1;             // row_ptr[n] when the host knows it (sizes shared-memory staging)
    // The cops' move graph when it differs from the robber's (row_ptr / col above), i.e. under
    // the stay-allowed rules; null = the same graph.  rrow_ptr / rcol and nbr always describe
    // the cops' moves.
    const uint32_t* cop_row_ptr = nullptr;
    const uint16_t* cop_col = nullptr;
    const uint32_t* cop_isolated = nullptr;
};

__host__ __device__ inline const uint32_t* cop_rows(const DevGraph& g) { return g.cop_row_ptr ? g.cop_row_ptr : g.row_ptr; }
__host__ __device__ inline const uint16_t* cop_cols(const DevGraph& g) { return g.cop_col ? g.cop_col : g.col; }
__host__ __device__ inline const uint32_t* cop_iso(const DevGraph& g) { return g.cop_isolated ? g.cop_isolated : g.isolated; }

// Everything one v1 solve's kernels touch.
struct V1Dev {
    DevGraph g;
    int k, cols, S;
    // words of dynamic shared memory past the last-column body's lane-group area where it may
    // stage the graph arrays its row tests read (0 = none)
    uint32_t and_stage_words = 0;
    uint32_t C;
    // a frontier with rows * push_ratio < C is pushed (kPushRatio; 0 = always push, ~0 = never)
    uint32_t push_ratio = kPushRatio;
    int fresh_last = 1;       // 0 = the last column always takes its general form
    const uint32_t* binom;    // [k][n + 1]: B[i][x] = C(n - x + k - 1 - i, k - i)
    const uint16_t* configs;  // [C][k]
    const uint32_t* hop;      // [n][rwp]: vertices exactly p robber moves from r
    uint8_t* table;
    uint32_t* marked;
    uint32_t* front;
    uint8_t* fflag;
    uint32_t* cand;           // [C][S][rwp]: push-mode OR of successor frontier rows
    // k = 3 dense cop turns: H1 rows [P][n][S][rwp], P = n(n+1)/2 pairs {x <= y}; H1[{x,y}][c]
    // = OR over z in N(c) of the frontier row of sort(x, y, z).  Null = the tuple-gathering pull.
    uint32_t* h1 = nullptr;
    uint32_t* cbits;          // [ceil(C / 32)]: bit C set = cand row C non-empty
    uint32_t* list;           // [cols][C]: the row lists of the columns' frontiers
    uint32_t* clist;          // [C]: ids of the non-empty cand rows (sync[1] of them)
    unsigned* sync;           // [2]: blocks done with the current prep, cand rows listed
    ColMeta* meta;            // [cols]
    unsigned long long* pass_new;
    unsigned int* err;
};

// Bookkeeping of a device-side pass loop: the history of pass counts, its length and capacity,
// and the WHILE node's condition.
struct LoopCtl {
    unsigned long long* hist;
    int* idx;
    int cap;
    cudaGraphConditionalHandle loop;
    // p = 1: the last column's prep is split between the cop turn's second launch (column 1's
    // flags and state) and the last column itself (the push form's candidate rows)
    int fused_prep1;
};

__host__ __device__ inline int round_words(int rw) { return rw <= 2 ? rw : (rw + 3) & ~3; }

// Raises a kernel's dynamic shared-memory limit to at least `bytes` and never lowers it.  The
// attribute belongs to the process, not to a stream or a solver: setting it to each launch's own
// size would let a smaller solve on another host thread shrink it under a larger one's launch,
// which then fails (or, for a kernel whose output is read without its own error check, leaves
// stale data).
inline cudaError_t raise_smem_limit(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<const void*, size_t> set;
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = set[kernel];
    if (bytes <= cur) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) cur = bytes;
    return e;
}

// Valid robber bits of word w of a row (the tail word of a row is partial).
__device__ __forceinline__ uint32_t valid_mask(int n, int w) {
    int lo = w * 32;
    if (lo >= n) return 0u;
    int left = n - lo;
    return left >= 32 ? 0xFFFFFFFFu : ((1u << left) - 1u);
}

// Lexicographic rank of a sorted multiset c[0..K) (the order of AuxGraph.h:160-176).
// Counting the multisets below c position by position and summing each position's range by
// the hockey-stick identity gives rank = sum_i B[i][c_{i-1}] - B[i][c_i] with c_{-1} = 0.
template <int K>
__device__ __forceinline__ uint32_t config_rank(const int (&c)[K], const uint32_t* __restrict__ B,
                                                int np1) {
    uint32_t r = 0;
    int prev = 0;
#pragma unroll
    for (int i = 0; i < K; ++i) {
        r += __ldg(&B[i * np1 + prev]) - __ldg(&B[i * np1 + c[i]]);
        prev = c[i];
    }
    return r;
}

template <int K>
__device__ __forceinline__ void sort_small(int (&c)[K]) {
#pragma unroll
    for (int i = 1; i < K; ++i) {
#pragma unroll
        for (int j = i; j > 0; --j) {
            int a = c[j - 1], b = c[j];
            c[j - 1] = min(a, b);
            c[j] = max(a, b);
        }
    }
}

template <typename T>
__device__ __forceinline__ T warp_or(T v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v |= __shfl_xor_sync(0xFFFFFFFFu, v, off);
    return v;
}

}  // namespace crgpu
