// crgpu_noalloc.cu - the v1 solve without any allocation, for callers that cannot allocate.
//
// Some callers cannot call cudaMalloc: code running under a memory budget owned by someone
// else (an arena or pool that must not grow), code that must not take the allocator's
// device-wide locks on a latency-critical path, or embedders that forbid the library from
// owning device memory.  cr_solve_v1_noalloc serves them: the caller passes the graph (host
// arrays) and the output table (device memory the caller owns), and every other buffer of
// the solve -- configuration table, marked and frontier planes, flags, push candidates,
// graph copies -- lives in one file-scope __device__ array of fixed size, kNoallocScratch
// bytes, that is part of the library image.
//
// Facts a caller has to know:
//   * every GPU that loads the library holds the scratch array (64 MiB) until the process
//     exits;
//   * the first call on a device looks the array's device address up with
//     cudaGetSymbolAddress (once per device, with that device current); make that first call
//     before any stream capture.  The address is kept for the process's life, so a
//     cudaDeviceReset (which destroys the context the address belongs to) makes it stale;
//   * it runs the general forms (unfused initializeCaptures, the tuple-gathering cop turn):
//     the fused first pass and the separable turn need tables beyond the area;
//   * all calls share the one array and leave the last call's contents in it: each call
//     clears what must start at zero, and two calls whose work overlaps on the GPU (other
//     streams, other host threads) race and corrupt each other;
//   * solves whose working set exceeds the array are refused with CR_ERR_LIMIT and a message
//     naming the bytes needed; no cudaMalloc, cudaFree, cudaMallocHost, event, graph or
//     stream is created, and no host heap memory is taken.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/crgpu.h"
#include "crgpu_internal.cuh"

namespace crgpu {
void launch_cop(const V1Dev& d, int col, int nx, int direct, int grid, cudaStream_t st, bool end = false);
void launch_and(const V1Dev& d, int col, bool p1, int grid, cudaStream_t st, const LoopCtl* loop = nullptr);
void launch_prep(const V1Dev& d, int col, int nx, int grid, cudaStream_t st);
void launch_init(const V1Dev& d, int grid, cudaStream_t st);
void launch_unrank(const uint32_t* B, int n, int k, uint32_t C, uint16_t* out, int grid, cudaStream_t st);
bool pull_supported(int S, int rwp);
size_t cop_smem_bytes(int S, int rwp);
size_t and_smem_bytes(int S, int rwp, int n);
}  // namespace crgpu

using namespace crgpu;

namespace {

constexpr size_t kNoallocScratch = 64ull << 20;  // bytes of the fixed scratch area
constexpr int kNoallocMaxN = 512;
constexpr int kNoallocMaxDevices = 64;

// The scratch area.  Host code must never pass `g_scratch` itself to a kernel: in host code
// the name is a stand-in, not a device address.  scratch_base() returns the real address.
static __device__ __align__(256) unsigned char g_scratch[kNoallocScratch];

std::mutex g_setup_mu;
unsigned char* g_scratch_dev[kNoallocMaxDevices] = {};

int scratch_base(int device, unsigned char** out, char* err, size_t err_len) {
    if (device < 0 || device >= kNoallocMaxDevices) {
        snprintf(err, err_len, "device %d outside 0..%d", device, kNoallocMaxDevices - 1);
        return CR_ERR_LIMIT;
    }
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_dev[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) {
            snprintf(err, err_len, "cudaGetSymbolAddress(scratch) failed: %s", cudaGetErrorString(e));
            return CR_ERR_CUDA;
        }
        g_scratch_dev[device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_dev[device];
    return CR_OK;
}

// Byte offsets of every buffer inside the scratch area (256-byte aligned).
struct Layout {
    size_t rp, col, rrp, rcol, cursor, nbr, iso, hop, rhop, binom, configs, marked, front, fflag,
        cand, cbits, list, clist, sync, meta, counters, err, total;
};

Layout plan(int n, size_t nnz, int k, int cols, uint64_t C, int rwp, int S) {
    Layout L;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t at = off;
        off += (bytes + 255) & ~size_t(255);
        return at;
    };
    const size_t ne = nnz ? nnz : 1;
    L.rp = take((size_t)(n + 1) * 4);
    L.col = take(ne * 2);
    L.rrp = take((size_t)(n + 1) * 4);
    L.rcol = take(ne * 2);
    L.cursor = take((size_t)n * 4);
    L.nbr = take((size_t)n * rwp * 4);
    L.iso = take((size_t)rwp * 4);
    L.hop = take((size_t)n * rwp * 4);
    L.rhop = take((size_t)n * rwp * 4);
    L.binom = take((size_t)k * (n + 1) * 4);
    L.configs = take(C * k * 2);
    L.marked = take((size_t)cols * C * rwp * 4);
    L.front = take((size_t)cols * C * S * rwp * 4);
    L.fflag = take((size_t)cols * C);
    L.cand = take(C * S * rwp * 4);
    L.cbits = take(cand_bits_bytes(C));
    L.list = take((size_t)cols * C * 4);
    L.clist = take(C * 4);
    L.sync = take(2 * sizeof(unsigned));
    L.meta = take(sizeof(ColMeta) * cols);
    L.counters = take(4 * sizeof(unsigned long long));
    L.err = take(sizeof(unsigned));
    L.total = off;
    return L;
}

uint64_t binom_small(int64_t n, int64_t k) {
    if (k < 0 || n < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    unsigned __int128 r = 1;
    for (int64_t i = 1; i <= k; ++i) r = r * (unsigned __int128)(n - i + 1) / (unsigned __int128)i;
    return r > (unsigned __int128)UINT64_MAX ? UINT64_MAX : (uint64_t)r;
}

// B[i][x] = C(n - x + k - 1 - i, k - i), the lexicographic rank table.
__global__ void k_na_binom(uint32_t* B, int n, int k) {
    const int np1 = n + 1;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < k * np1; t += gridDim.x * blockDim.x) {
        const int i = t / np1, x = t - i * np1;
        const long long top = (long long)n - x + k - 1 - i, kk = k - i;
        unsigned long long r = 1;
        if (kk > top) r = 0;
        else
            for (long long j = 1; j <= kk; ++j) r = r * (unsigned long long)(top - j + 1) / (unsigned long long)j;
        B[t] = (uint32_t)r;
    }
}

// In-degree counts, out-neighbour masks and the isolated-vertex mask.
__global__ void k_na_graph(const uint32_t* rp, const uint16_t* col, int n, int rwp, uint32_t* indeg,
                           uint32_t* nbr, uint32_t* iso) {
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
        if (rp[u + 1] == rp[u]) atomicOr(&iso[u >> 5], 1u << (u & 31));
        for (uint32_t e = rp[u]; e < rp[u + 1]; ++e) {
            const int v = col[e];
            atomicAdd(&indeg[v], 1u);
            nbr[(size_t)u * rwp + (v >> 5)] |= 1u << (v & 31);  // row u is this thread's
        }
    }
}

// Exclusive scan of the in-degrees into rrp (n <= 512: one thread is plenty).
__global__ void k_na_scan(uint32_t* cursor_in_out, uint32_t* rrp, int n) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    uint32_t run = 0;
    for (int v = 0; v < n; ++v) {
        rrp[v] = run;
        run += cursor_in_out[v];
        cursor_in_out[v] = rrp[v];
    }
    rrp[n] = run;
}

// In-neighbour lists (their order is irrelevant: push mode only ORs over them).
__global__ void k_na_fill(const uint32_t* rp, const uint16_t* col, int n, uint32_t* cursor, uint16_t* rcol) {
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x)
        for (uint32_t e = rp[u]; e < rp[u + 1]; ++e) rcol[atomicAdd(&cursor[col[e]], 1u)] = (uint16_t)u;
}

// Exact-p-hop vertex sets (k_cops_visibility.cpp:245-262, robber self-edges off).
__global__ void k_na_hop(const uint32_t* nbr, int n, int rwp, int p, uint32_t* hop) {
    constexpr int W = kNoallocMaxN / 32;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        uint32_t cur[W], nxt[W];
        for (int w = 0; w < W; ++w) cur[w] = 0u;
        cur[r >> 5] = 1u << (r & 31);
        for (int s = 0; s < p; ++s) {
            for (int w = 0; w < W; ++w) nxt[w] = 0u;
            for (int w = 0; w < rwp; ++w) {
                uint32_t b = cur[w];
                while (b) {
                    const int v = w * 32 + __ffs(b) - 1;
                    b &= b - 1;
                    for (int q = 0; q < rwp; ++q) nxt[q] |= nbr[(size_t)v * rwp + q];
                }
            }
            for (int w = 0; w < W; ++w) cur[w] = nxt[w];
        }
        for (int w = 0; w < rwp; ++w) hop[(size_t)r * rwp + w] = cur[w];
    }
}

// Transposed hop masks: bit r of row u iff u is in hop(r).
__global__ void k_na_rhop(const uint32_t* hop, int n, int rwp, uint32_t* rhop) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x)
        for (int w = 0; w < rwp; ++w) {
            uint32_t b = hop[(size_t)r * rwp + w];
            while (b) {
                const int u = w * 32 + __ffs(b) - 1;
                b &= b - 1;
                atomicOr(&rhop[(size_t)u * rwp + (r >> 5)], 1u << (r & 31));
            }
        }
}

int fail(char* err, size_t err_len, int code, const char* msg) {
    if (err && err_len) snprintf(err, err_len, "%s", msg);
    return code;
}

#define NA_CUDA(call)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            if (err && err_len) snprintf(err, err_len, "%s: %s", #call, cudaGetErrorString(e_)); \
            return CR_ERR_CUDA;                                                              \
        }                                                                                    \
    } while (0)

}  // namespace

extern "C" int cr_solve_v1_noalloc(const cr_graph* g, int32_t k, int32_t p, void* stream,
                                   uint8_t* states_dev, size_t states_bytes, uint64_t* pass_counts,
                                   int32_t cap, int32_t* passes, uint64_t* base_captures,
                                   char* err, size_t err_len) {
    if (err && err_len) err[0] = '\0';
    if (!g || !g->row_ptr || !states_dev || !pass_counts || !passes || cap <= 0)
        return fail(err, err_len, CR_ERR_INVALID, "graph, output table, pass_counts and passes are required");
    const int n = g->n;
    if (n <= 0) return fail(err, err_len, CR_ERR_INVALID, "Graph is empty or failed to load.");
    if (n > kNoallocMaxN) return fail(err, err_len, CR_ERR_LIMIT, "the no-allocation solve handles at most 512 vertices");
    if (k <= 0 || k > CR_MAX_K) return fail(err, err_len, CR_ERR_LIMIT, "k outside 1..4");
    if (p <= 0 || p > 63) return fail(err, err_len, CR_ERR_INVALID, "p outside 1..63");
    const size_t nnz = g->row_ptr[n];
    if (nnz && !g->col_idx) return fail(err, err_len, CR_ERR_INVALID, "graph arrays missing");
    for (int v = 0; v < n; ++v)
        if (g->row_ptr[v + 1] < g->row_ptr[v]) return fail(err, err_len, CR_ERR_INVALID, "row_ptr not monotone");
    for (size_t e = 0; e < nnz; ++e)
        if (g->col_idx[e] >= n) return fail(err, err_len, CR_ERR_INVALID, "neighbour index out of range");
    const uint64_t C = binom_small((int64_t)n + k - 1, k);
    if (C == 0 || C >= (1ull << 32)) return fail(err, err_len, CR_ERR_LIMIT, "configuration count out of range");
    const int cols = 2 * p, rw = (n + 31) / 32, rwp = round_words(rw);
    const size_t table_bytes = C * (size_t)n * cols;
    if (states_bytes < table_bytes) {
        if (err && err_len) snprintf(err, err_len, "output table holds %zu of %zu bytes", states_bytes, table_bytes);
        return CR_ERR_INVALID;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int device = 0, sms = 1;
    NA_CUDA(cudaGetDevice(&device));
    NA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    unsigned char* base = nullptr;
    int rc = scratch_base(device, &base, err, err_len);
    if (rc) return rc;

    for (int S = 2; S <= 8; S *= 2) {
        if (!pull_supported(S, rwp)) return fail(err, err_len, CR_ERR_LIMIT, "rows too wide for the warp layout");
        const Layout L = plan(n, nnz, k, cols, C, rwp, S);
        if (L.total > kNoallocScratch) {
            if (err && err_len)
                snprintf(err, err_len, "solve needs %zu bytes of scratch; the fixed area holds %zu (64 MiB)",
                         L.total, kNoallocScratch);
            return CR_ERR_LIMIT;
        }
        // everything the solve reads before writing starts at zero
        NA_CUDA(cudaMemsetAsync(base, 0, L.total, st));
        NA_CUDA(cudaMemcpyAsync(base + L.rp, g->row_ptr, (size_t)(n + 1) * 4, cudaMemcpyHostToDevice, st));
        if (nnz) NA_CUDA(cudaMemcpyAsync(base + L.col, g->col_idx, nnz * 2, cudaMemcpyHostToDevice, st));
        V1Dev d;
        d.g.n = n;
        d.g.rw = rw;
        d.g.rwp = rwp;
        d.g.row_ptr = reinterpret_cast<const uint32_t*>(base + L.rp);
        d.g.col = reinterpret_cast<const uint16_t*>(base + L.col);
        d.g.rrow_ptr = reinterpret_cast<const uint32_t*>(base + L.rrp);
        d.g.rcol = reinterpret_cast<const uint16_t*>(base + L.rcol);
        d.g.nbr = reinterpret_cast<const uint32_t*>(base + L.nbr);
        d.g.isolated = reinterpret_cast<const uint32_t*>(base + L.iso);
        d.g.rhop = reinterpret_cast<const uint32_t*>(base + L.rhop);
        d.g.nnz = (int)nnz;   // lets the last column stage the graph in shared memory
        int maxdeg = 0;
        for (int v = 0; v < n; ++v) maxdeg = maxdeg > (int)(g->row_ptr[v + 1] - g->row_ptr[v]) ? maxdeg : (int)(g->row_ptr[v + 1] - g->row_ptr[v]);
        d.g.maxdeg = maxdeg;
        d.k = k;
        d.cols = cols;
        d.S = S;
        d.C = (uint32_t)C;
        d.binom = reinterpret_cast<const uint32_t*>(base + L.binom);
        d.configs = reinterpret_cast<const uint16_t*>(base + L.configs);
        d.hop = reinterpret_cast<const uint32_t*>(base + L.hop);
        d.table = states_dev;
        d.marked = reinterpret_cast<uint32_t*>(base + L.marked);
        d.front = reinterpret_cast<uint32_t*>(base + L.front);
        d.fflag = base + L.fflag;
        d.cand = reinterpret_cast<uint32_t*>(base + L.cand);
        d.cbits = reinterpret_cast<uint32_t*>(base + L.cbits);
        d.list = reinterpret_cast<uint32_t*>(base + L.list);
        d.clist = reinterpret_cast<uint32_t*>(base + L.clist);
        d.sync = reinterpret_cast<unsigned*>(base + L.sync);
        d.meta = reinterpret_cast<ColMeta*>(base + L.meta);
        d.pass_new = reinterpret_cast<unsigned long long*>(base + L.counters);
        d.err = reinterpret_cast<unsigned*>(base + L.err);

        const int gsmall = (int)(C + 255) / 256 < sms * 4 ? (int)((C + 255) / 256) : sms * 4;
        const int gcop = (int)((C + 7) / 8) < sms * 4 ? (int)((C + 7) / 8) : sms * 4;
        uint32_t* cursor = reinterpret_cast<uint32_t*>(base + L.cursor);
        k_na_binom<<<8, 256, 0, st>>>(reinterpret_cast<uint32_t*>(base + L.binom), n, k);
        k_na_graph<<<4, 256, 0, st>>>(d.g.row_ptr, d.g.col, n, rwp, cursor,
                                      reinterpret_cast<uint32_t*>(base + L.nbr),
                                      reinterpret_cast<uint32_t*>(base + L.iso));
        k_na_scan<<<1, 1, 0, st>>>(cursor, reinterpret_cast<uint32_t*>(base + L.rrp), n);
        k_na_fill<<<4, 256, 0, st>>>(d.g.row_ptr, d.g.col, n, cursor, reinterpret_cast<uint16_t*>(base + L.rcol));
        k_na_hop<<<4, 128, 0, st>>>(d.g.nbr, n, rwp, p, reinterpret_cast<uint32_t*>(base + L.hop));
        k_na_rhop<<<4, 128, 0, st>>>(d.hop, n, rwp, reinterpret_cast<uint32_t*>(base + L.rhop));
        launch_unrank(d.binom, n, k, (uint32_t)C, reinterpret_cast<uint16_t*>(base + L.configs),
                      gsmall > 0 ? gsmall : 1, st);
        NA_CUDA(cudaGetLastError());

        // initializeCaptures (k_cops_visibility.cpp:85-127)
        ColMeta meta[126];
        for (int c = 0; c < cols; ++c) meta[c] = ColMeta{0, kEmptyLo, -1, 0, 0, 0, 0, 0};
        const int rows = C < 0x7FFFFFFFull ? (int)C : 0x7FFFFFFF;
        meta[0] = ColMeta{0, 0, 0, 1, rows, 0, -1, 0};
        meta[1] = ColMeta{0, 0, 0, 0, rows, 1, -1, 0};
        NA_CUDA(cudaMemcpyAsync(d.meta, meta, sizeof(ColMeta) * cols, cudaMemcpyHostToDevice, st));
        NA_CUDA(cudaMemsetAsync(states_dev, kUnmarked, table_bytes, st));
        launch_init(d, gsmall > 0 ? gsmall : 1, st);
        NA_CUDA(cudaGetLastError());
        unsigned long long caps = 0;
        NA_CUDA(cudaMemcpyAsync(&caps, d.pass_new, sizeof(caps), cudaMemcpyDeviceToHost, st));
        NA_CUDA(cudaStreamSynchronize(st));

        // mainLoop (k_cops_visibility.cpp:142-296), one column producer after another
        int np = 0;
        bool overflow = false;
        for (;;) {
            for (int col = 0; col < cols; ++col) {
                const int nx = (col + 1) % cols;
                launch_prep(d, col, nx, gsmall > 0 ? gsmall : 1, st);
                if (col % 2 == 0) launch_cop(d, col, nx, 0, gcop > 0 ? gcop : 1, st);
                else if (col < cols - 1) launch_cop(d, col, nx, 1, gcop > 0 ? gcop : 1, st);
                else launch_and(d, col, p == 1, gcop > 0 ? gcop : 1, st);
            }
            NA_CUDA(cudaGetLastError());
            unsigned long long found = 0;
            unsigned bits = 0;
            NA_CUDA(cudaMemcpyAsync(&found, d.pass_new, sizeof(found), cudaMemcpyDeviceToHost, st));
            NA_CUDA(cudaMemcpyAsync(&bits, d.err, sizeof(bits), cudaMemcpyDeviceToHost, st));
            NA_CUDA(cudaStreamSynchronize(st));
            if (bits & kErrRank) return fail(err, err_len, CR_ERR_INTERNAL, "successor rank out of range");
            if (bits & kErrSlot) { overflow = true; break; }
            if (np >= cap) return fail(err, err_len, CR_ERR_BUDGET, "pass_counts capacity reached before the fixed point");
            pass_counts[np++] = found;
            if (found == 0) break;
        }
        if (overflow) continue;  // value range wider than S slots: redo with twice as many
        *passes = np;
        if (base_captures) *base_captures = caps;
        return CR_OK;
    }
    return fail(err, err_len, CR_ERR_INTERNAL, "frontier value range exceeds 8 slots");
}
