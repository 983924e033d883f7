// crgpu_api.cu - the C ABI of include/crgpu.h: contexts, graph parsing, the v1 solve
// schedule, verdict, table read-out and the table-file writer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/crgpu.h"
#include "crgpu_internal.cuh"
#include "crgpu_ctx.h"
#include "crgpu_v2.h"

namespace crgpu {
void launch_cop(const V1Dev& d, int col, int nx, int direct, int grid, cudaStream_t st, bool end = false);
void launch_and(const V1Dev& d, int col, bool p1, int grid, cudaStream_t st, const LoopCtl* loop = nullptr);
void launch_prep(const V1Dev& d, int col, int nx, int grid, cudaStream_t st);
void launch_init(const V1Dev& d, int grid, cudaStream_t st);
void launch_init_pass1(const V1Dev& d, int num_sms, cudaStream_t st);
void launch_list_compact(const V1Dev& d, int col, int num_sms, cudaStream_t st);
void launch_marks_from_table(const uint8_t* table, uint32_t C, int n, int cols, int rwp, uint32_t* marked,
                             int grid, cudaStream_t st);
void launch_game(const uint8_t* table, const uint16_t* configs, const unsigned long long* heads,
                 const unsigned long long* trans, const uint32_t* rp, const uint16_t* adj, int n, int k,
                 long long best, int cap, long long* out_c, int* out_r, int* count, int* captured,
                 cudaStream_t st);
void launch_loop_enter(const V1Dev& d, const LoopCtl& c, int grid, cudaStream_t st);
void launch_verdict(const V1Dev& d, int cols, unsigned long long* best, int grid, cudaStream_t st);
void launch_popcount(const uint32_t* plane, size_t words, unsigned long long* out, int grid,
                     cudaStream_t st);
int max_cop_blocks_per_sm(int k, int rwp, int S);
bool pull_supported(int S, int rwp);
int cop_launches(int direct);
int cop_launches_k(int direct, int k, bool sep);
size_t cop_smem_bytes(int S, int rwp);
size_t and_smem_bytes(int S, int rwp, int n);
void launch_unrank(const uint32_t* B, int n, int k, uint32_t C, uint16_t* out, int grid, cudaStream_t st);
int trans_cap(int k, int maxdeg);
void launch_trans(int k, const uint16_t* configs, uint32_t C, int n, const uint32_t* rp,
                  const uint16_t* adj, const uint32_t* B, int cap, unsigned long long* counts,
                  const unsigned long long* heads, unsigned long long* data, unsigned int* err,
                  int grid, cudaStream_t st);
void launch_scan(const unsigned long long* in, unsigned long long* out, uint32_t C, cudaStream_t st);
void launch_digest(const uint8_t* table, size_t bytes, unsigned long long* out, int grid, cudaStream_t st);
}  // namespace crgpu

using namespace crgpu;

// Per-solve state.  Host copies of the graph are kept for the hop masks and file output.
struct cr_solver {
    cr_context* ctx = nullptr;
    int n = 0, k = 0, p = 0, rules = CR_RULES_V1, cols = 0, rw = 0, rwp = 0, S = 2;
    uint64_t C = 0;
    int maxdeg = 0;
    std::vector<uint32_t> h_rp;       // the robber's moves (with self-loops under CR_ROBBER_STAY)
    std::vector<uint16_t> h_col;
    std::vector<uint32_t> h_crp;      // the cops' moves (with self-loops under CR_COP_STAY)
    std::vector<uint16_t> h_ccol;
    bool cop_stay = false, robber_stay = false;
    int cop_maxdeg = 0;
    uint32_t forms = CR_FORMS_ALL;    // cr_solver_set_forms
    uint32_t* d_crp = nullptr;        // set only when the two move graphs differ
    uint16_t* d_ccol = nullptr;
    uint32_t* d_ciso = nullptr;
    std::vector<uint32_t> h_binom;
    // device
    uint32_t* d_rp = nullptr;
    uint16_t* d_col = nullptr;
    uint32_t* d_binom = nullptr;
    uint16_t* d_configs = nullptr;
    uint32_t* d_hop = nullptr;
    uint8_t* d_table = nullptr;
    uint32_t* d_marked = nullptr;
    uint32_t* d_front = nullptr;
    uint8_t* d_fflag = nullptr;
    uint32_t* d_cand = nullptr;
    uint32_t* d_h1 = nullptr;   // k = 3: H1 rows of the separable dense cop turn
    uint32_t* d_cbits = nullptr;      // push-mode candidate bitmap
    uint32_t* d_list = nullptr;       // [cols][C] row lists of the frontiers
    uint32_t* d_clist = nullptr;      // [C] push-mode candidate list
    unsigned* d_sync = nullptr;       // [2] prep's block count, candidate count
    uint32_t* d_rrp = nullptr;
    uint16_t* d_rcol = nullptr;
    uint32_t* d_nbr = nullptr;
    uint32_t* d_iso = nullptr;
    uint32_t* d_rhop = nullptr;
    uint8_t* d_cover = nullptr;   // first-pass neighbour-slot masks (p = 1, max degree <= 32)
    int cover_w = 0, npad = 0;
    ColMeta* d_meta = nullptr;
    unsigned long long* d_counters = nullptr;  // [0] pass_new, [1] verdict key, [2] scratch
    unsigned int* d_err = nullptr;
    unsigned long long* d_heads = nullptr;
    unsigned long long* d_trans = nullptr;
    uint64_t n_trans = 0;
    // pinned read-back slots: [0..3] counters, [4..4+kPinHist) the pass history, then its
    // length and the error bits
    unsigned long long* h_pinned = nullptr;
    cudaGraphExec_t pass_graph = nullptr;
    // mainLoop on the device: a graph whose WHILE node replays one pass until a pass finds
    // nothing; the pass counts land in d_hist, their number in d_hist_n
    cudaGraphExec_t run_graph = nullptr;
    unsigned long long* d_hist = nullptr;
    int* d_hist_n = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, evc0 = nullptr, evc1 = nullptr;
    // phase state
    bool initialized = false;
    bool finished = false;
    // p = 1: initializeCaptures is folded into the first pass (one sweep writes the table);
    // set between cr_solver_init and that pass, and undone by materialize_init() when the
    // post-initializeCaptures state is read first
    bool init_pending = false;
    // small solves launch each pass's kernels directly: capturing and instantiating a graph
    // costs more than it saves over a handful of short passes, and contends for the CUDA driver
    // when many solves run side by side (the solve server)
    bool small = false;
    uint64_t base_caps = 0;
    std::vector<uint64_t> pass_counts;
    cr_solve_stats stats{};
    int grid_cop = 1, grid_small = 1;
    crgpu::V2Solver* v2 = nullptr;
};

static int fail(cr_context* ctx, int code, const char* fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->err = buf;
    }
    return code;
}

#define CR_CUDA(ctx, call)                                                                  \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail((ctx), CR_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

static constexpr int kPinHist = 64;   // pass counts read back with the pass loop's end

static uint64_t binom_u64(int64_t n, int64_t k) {
    if (k < 0 || n < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    unsigned __int128 r = 1;
    for (int64_t i = 1; i <= k; ++i) {
        r = r * (unsigned __int128)(n - i + 1) / (unsigned __int128)i;
        if (r > (unsigned __int128)UINT64_MAX) return UINT64_MAX;
    }
    return (uint64_t)r;
}

extern "C" {

int cr_context_create(int32_t device, void* stream, cr_context** out) {
    if (!out) return CR_ERR_INVALID;
    *out = nullptr;
    cr_context* c = new (std::nothrow) cr_context();
    if (!c) return CR_ERR_NOMEM;
    c->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) {
        if (stream) {
            c->stream = (cudaStream_t)stream;
        } else {
            e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
            c->own_stream = true;
        }
    }
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        delete c;
        return CR_ERR_CUDA;
    }
    *out = c;
    return CR_OK;
}

int cr_context_destroy(cr_context* ctx) {
    if (!ctx) return CR_OK;
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    cudaSetDevice(ctx->device);
    ctx->cache.clear();
    delete ctx;
    return CR_OK;
}

const char* cr_context_last_error(const cr_context* ctx) { return ctx ? ctx->err.c_str() : ""; }

int cr_context_set_cache_limit(cr_context* ctx, uint64_t bytes) {
    if (!ctx) return CR_ERR_INVALID;
    CR_CUDA(ctx, cudaSetDevice(ctx->device));
    ctx->cache.set_limit(bytes);
    return CR_OK;
}

int cr_context_set_profiling(cr_context* ctx, int32_t on) {
    if (!ctx) return CR_ERR_INVALID;
    ctx->profiling = on != 0;
    return CR_OK;
}

int cr_graph_parse(const char* text, size_t len, int32_t* n_out, uint32_t* row_ptr,
                   uint16_t* col_idx, size_t col_cap, size_t* nnz_out) {
    // Graph::Graph (lib/src/Graph.cpp:26-70): N = first-line width; '0'/'1' fill row-major;
    // '\n' advances the row only after a digit; '-' ends the matrix; anything else is skipped.
    if (!n_out || !nnz_out || (!text && len)) return CR_ERR_INVALID;
    size_t n = 0;
    while (n < len && text[n] != '\n' && text[n] != '\r' && text[n] != '-') ++n;
    if (n > CR_MAX_N) return CR_ERR_LIMIT;
    *n_out = (int32_t)n;
    std::vector<uint8_t> m(n * n, 0);
    size_t row = 0, col = 0;
    for (size_t i = 0; i < len && n; ++i) {
        char c = text[i];
        if (c == '-') break;
        if (c == '0' || c == '1') {
            if (row < n && col < n) m[row * n + col] = (uint8_t)(c == '1');
            ++col;
        } else if (c == '\n') {
            if (col > 0) { ++row; col = 0; }
        }
    }
    size_t nnz = 0;
    for (uint8_t x : m) nnz += x;
    *nnz_out = nnz;
    if (!row_ptr) return CR_OK;
    if (!col_idx && nnz) return CR_ERR_INVALID;
    if (col_cap < nnz) return CR_ERR_INVALID;
    size_t e = 0;
    row_ptr[0] = 0;
    for (size_t r = 0; r < n; ++r) {
        for (size_t c = 0; c < n; ++c)
            if (m[r * n + c]) col_idx[e++] = (uint16_t)c;
        row_ptr[r + 1] = (uint32_t)e;
    }
    return CR_OK;
}

static int slots_for(int n) { (void)n; return 2; }

// H1 rows of the separable dense cop turn (k = 3): every pair {x <= y} times every vertex,
// one frontier row each; about 3/8 of the table's bytes.  0 when the turn keeps the
// tuple-gathering form.
static uint64_t h1_bytes(int n, int k, int S, int rwp) {
    if (k != 3 || !pull_supported(S, rwp)) return 0;
    return (uint64_t)n * (n + 1) / 2 * n * S * rwp * 4;
}

static void layout(int n, int k, int p, int rules, int S, uint64_t* C, int* cols, int* rw, int* rwp) {
    *C = binom_u64((int64_t)n + k - 1, k);
    *cols = rules == CR_RULES_V2 ? 1 : 2 * p;
    *rw = (n + 31) / 32;
    *rwp = round_words(*rw);
    (void)S;
}

uint64_t cr_solver_footprint(int32_t n, int32_t k, int32_t p, int32_t rules) {
    if (n <= 0 || k <= 0 || p <= 0) return 0;
    if (rules == CR_RULES_V2) return crgpu::v2_footprint(n, k, p);
    uint64_t C;
    int cols, rw, rwp;
    const int S = slots_for(n);
    layout(n, k, p, rules, S, &C, &cols, &rw, &rwp);
    uint64_t b = C * (uint64_t)n * cols;                 // table
    b += (uint64_t)cols * C * rwp * 4;                   // marked
    b += (uint64_t)cols * C * S * rwp * 4;               // frontiers
    b += C * S * rwp * 4 + cand_bits_bytes(C) + C * 4;   // push-mode candidate rows, bitmap, list
    b += (uint64_t)cols * C * 4 + 2 * sizeof(unsigned);  // frontier row lists, prep/list counters
    b += h1_bytes(n, k, S, rwp);                         // separable dense cop turn (k = 3)
    b += (uint64_t)cols * C;                             // flags
    b += C * (uint64_t)k * 2;                            // configs
    b += (uint64_t)n * rwp * 4 * 3 + (uint64_t)k * (n + 1) * 4 + (1u << 16);
    if (cols == 2) b += 2ull * n * (uint64_t)((n + 7) & ~7) * 4;   // first-pass cover masks
    b += (1u << 16) * 8ull + 256;                                 // device pass-loop history
    return b;
}

static void free_v1(cr_solver* s) {
    if (s->pass_graph) cudaGraphExecDestroy(s->pass_graph);
    s->pass_graph = nullptr;
    if (s->run_graph) cudaGraphExecDestroy(s->run_graph);
    s->run_graph = nullptr;
    if (s->d_hist) cudaFree(s->d_hist);
    if (s->d_hist_n) cudaFree(s->d_hist_n);
    s->d_hist = nullptr;
    s->d_hist_n = nullptr;
    void* ptrs[] = {s->d_rp, s->d_col, s->d_binom, s->d_configs, s->d_hop, s->d_table,
                    s->d_marked, s->d_front, s->d_fflag, s->d_meta, s->d_counters, s->d_err,
                    s->d_heads, s->d_trans, s->d_cand, s->d_cbits, s->d_list, s->d_clist, s->d_sync,
                    s->d_rrp, s->d_rcol, s->d_nbr, s->d_iso, s->d_rhop, s->d_cover,
                    s->d_crp, s->d_ccol, s->d_ciso, s->d_h1};
    for (void* q : ptrs) s->ctx->cache.put(q);   // the context keeps large blocks for reuse
    s->d_rp = nullptr; s->d_col = nullptr; s->d_binom = nullptr; s->d_configs = nullptr;
    s->d_hop = nullptr; s->d_table = nullptr; s->d_marked = nullptr; s->d_front = nullptr;
    s->d_fflag = nullptr; s->d_meta = nullptr; s->d_counters = nullptr; s->d_err = nullptr;
    s->d_heads = nullptr; s->d_trans = nullptr; s->d_cand = nullptr; s->d_cbits = nullptr;
    s->d_list = nullptr; s->d_clist = nullptr; s->d_sync = nullptr;
    s->d_rrp = nullptr; s->d_rcol = nullptr; s->d_nbr = nullptr; s->d_iso = nullptr; s->d_rhop = nullptr;
    s->d_cover = nullptr;
    s->d_crp = nullptr; s->d_ccol = nullptr; s->d_ciso = nullptr; s->d_h1 = nullptr;
    if (s->h_pinned) cudaFreeHost(s->h_pinned);
    s->h_pinned = nullptr;
    cudaEvent_t evs[] = {s->ev0, s->ev1, s->evc0, s->evc1};
    for (cudaEvent_t e : evs)
        if (e) cudaEventDestroy(e);
    s->ev0 = s->ev1 = s->evc0 = s->evc1 = nullptr;
}

static V1Dev dev_view(const cr_solver* s) {
    V1Dev d;
    d.g.n = s->n;
    d.g.rw = s->rw;
    d.g.rwp = s->rwp;
    d.g.row_ptr = s->d_rp;
    d.g.col = s->d_col;
    d.g.rrow_ptr = s->d_rrp;
    d.g.rcol = s->d_rcol;
    d.g.nbr = s->d_nbr;
    d.g.isolated = s->d_iso;
    d.g.rhop = s->d_rhop;
    d.g.maxdeg = s->maxdeg;
    d.g.cover = s->d_cover;
    d.g.cover_w = s->cover_w;
    d.g.npad = s->npad;
    d.g.nnz = (int)s->h_col.size();
    d.g.cop_row_ptr = s->d_crp;
    d.g.cop_col = s->d_ccol;
    d.g.cop_isolated = s->d_ciso;
    d.k = s->k;
    d.cols = s->cols;
    d.S = s->S;
    d.C = (uint32_t)s->C;
    d.binom = s->d_binom;
    d.configs = s->d_configs;
    d.hop = s->d_hop;
    d.table = s->d_table;
    d.marked = s->d_marked;
    d.front = s->d_front;
    d.fflag = s->d_fflag;
    d.cand = s->d_cand;
    d.h1 = s->d_h1;
    d.cbits = s->d_cbits;
    // forms switched off: no pair rows (the tuple pull), a push ratio that always or never
    // pushes, the last column's general form
    if (!(s->forms & CR_FORM_SEPARABLE)) d.h1 = nullptr;
    if (!(s->forms & CR_FORM_PULL)) d.push_ratio = 0u;
    else if (!(s->forms & CR_FORM_PUSH)) d.push_ratio = 0xFFFFFFFFu;
    d.fresh_last = (s->forms & CR_FORM_FRESH_LAST) ? 1 : 0;
    d.list = s->d_list;
    d.clist = s->d_clist;
    d.sync = s->d_sync;
    d.meta = s->d_meta;
    d.pass_new = s->d_counters;
    d.err = s->d_err;
    return d;
}

// Exact-p-hop vertex sets (k_cops_visibility.cpp:245-262, robber self-edges off).
static std::vector<uint32_t> hop_masks(const cr_solver* s) {
    std::vector<uint32_t> hop((size_t)s->n * s->rwp, 0);
    std::vector<uint8_t> cur(s->n), nxt(s->n);
    for (int r = 0; r < s->n; ++r) {
        std::fill(cur.begin(), cur.end(), 0);
        cur[r] = 1;
        for (int step = 0; step < s->p; ++step) {
            std::fill(nxt.begin(), nxt.end(), 0);
            for (int v = 0; v < s->n; ++v)
                if (cur[v])
                    for (uint32_t e = s->h_rp[v]; e < s->h_rp[v + 1]; ++e) nxt[s->h_col[e]] = 1;
            cur.swap(nxt);
        }
        for (int v = 0; v < s->n; ++v)
            if (cur[v]) hop[(size_t)r * s->rwp + (v >> 5)] |= 1u << (v & 31);
    }
    return hop;
}

static int alloc_v1(cr_solver* s) {
    cr_context* ctx = s->ctx;
    const size_t C = s->C;
    CR_CUDA(ctx, ctx->cache.get((void**)&s->d_table, C * s->n * s->cols));
    CR_CUDA(ctx, ctx->cache.get((void**)&s->d_marked, (size_t)s->cols * C * s->rwp * 4));
    CR_CUDA(ctx, ctx->cache.get((void**)&s->d_front, (size_t)s->cols * C * s->S * s->rwp * 4));
    CR_CUDA(ctx, ctx->cache.get((void**)&s->d_fflag, (size_t)s->cols * C));
    CR_CUDA(ctx, cudaMalloc(&s->d_meta, sizeof(ColMeta) * s->cols));
    CR_CUDA(ctx, ctx->cache.get((void**)&s->d_cand, C * s->S * s->rwp * 4));
    CR_CUDA(ctx, ctx->cache.get((void**)&s->d_cbits, cand_bits_bytes(C)));
    CR_CUDA(ctx, ctx->cache.get((void**)&s->d_list, (size_t)s->cols * C * 4));
    CR_CUDA(ctx, ctx->cache.get((void**)&s->d_clist, C * 4));
    CR_CUDA(ctx, cudaMalloc(&s->d_sync, 2 * sizeof(unsigned)));
    CR_CUDA(ctx, cudaMemsetAsync(s->d_cand, 0, C * s->S * s->rwp * 4, ctx->stream));
    CR_CUDA(ctx, cudaMemsetAsync(s->d_cbits, 0, cand_bits_bytes(C), ctx->stream));
    if (const uint64_t hb = h1_bytes(s->n, s->k, s->S, s->rwp)) CR_CUDA(ctx, ctx->cache.get((void**)&s->d_h1, hb));
    CR_CUDA(ctx, cudaMalloc(&s->d_hop, (size_t)s->n * s->rwp * 4));
    std::vector<uint32_t> hop = hop_masks(s);
    CR_CUDA(ctx, cudaMemcpyAsync(s->d_hop, hop.data(), hop.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    // transposed hop masks: bit r of row u iff u in hop(r)
    std::vector<uint32_t> rhop(hop.size(), 0);
    for (int r = 0; r < s->n; ++r)
        for (int u = 0; u < s->n; ++u)
            if ((hop[(size_t)r * s->rwp + (u >> 5)] >> (u & 31)) & 1u)
                rhop[(size_t)u * s->rwp + (r >> 5)] |= 1u << (r & 31);
    CR_CUDA(ctx, cudaMalloc(&s->d_rhop, rhop.size() * 4));
    CR_CUDA(ctx, cudaMemcpyAsync(s->d_rhop, rhop.data(), rhop.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    // the cops' out-neighbour masks (capture-seed closed form) and their in-neighbour CSR
    // (push mode), both of the cops' move graph
    const std::vector<uint32_t>& crp = s->h_crp;
    const std::vector<uint16_t>& ccol = s->h_ccol;
    std::vector<uint32_t> nbr((size_t)s->n * s->rwp, 0);
    std::vector<uint32_t> rrp(s->n + 1, 0);
    for (uint32_t e = 0; e < ccol.size(); ++e) rrp[ccol[e] + 1]++;
    for (int v = 0; v < s->n; ++v) rrp[v + 1] += rrp[v];
    std::vector<uint16_t> rcol(std::max<size_t>(ccol.size(), 1));
    std::vector<uint32_t> fill(rrp.begin(), rrp.end() - 1);
    for (int u = 0; u < s->n; ++u)
        for (uint32_t e = crp[u]; e < crp[u + 1]; ++e) {
            const int v = ccol[e];
            nbr[(size_t)u * s->rwp + (v >> 5)] |= 1u << (v & 31);
            rcol[fill[v]++] = (uint16_t)u;  // in-neighbours of v, ascending u
        }
    // robbers without a move (the last column's vacuous AND), cops without a move
    std::vector<uint32_t> iso(s->rwp, 0), ciso(s->rwp, 0);
    for (int v = 0; v < s->n; ++v) {
        if (s->h_rp[v + 1] == s->h_rp[v]) iso[v >> 5] |= 1u << (v & 31);
        if (crp[v + 1] == crp[v]) ciso[v >> 5] |= 1u << (v & 31);
    }
    if (s->cop_stay != s->robber_stay) {
        CR_CUDA(ctx, cudaMalloc(&s->d_crp, crp.size() * 4));
        CR_CUDA(ctx, cudaMalloc(&s->d_ccol, std::max<size_t>(ccol.size(), 1) * 2));
        CR_CUDA(ctx, cudaMalloc(&s->d_ciso, ciso.size() * 4));
        CR_CUDA(ctx, cudaMemcpyAsync(s->d_crp, crp.data(), crp.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
        if (!ccol.empty())
            CR_CUDA(ctx, cudaMemcpyAsync(s->d_ccol, ccol.data(), ccol.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
        CR_CUDA(ctx, cudaMemcpyAsync(s->d_ciso, ciso.data(), ciso.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    }
    CR_CUDA(ctx, cudaMalloc(&s->d_iso, iso.size() * 4));
    CR_CUDA(ctx, cudaMemcpyAsync(s->d_iso, iso.data(), iso.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    CR_CUDA(ctx, cudaMalloc(&s->d_nbr, nbr.size() * 4));
    CR_CUDA(ctx, cudaMalloc(&s->d_rrp, rrp.size() * 4));
    CR_CUDA(ctx, cudaMalloc(&s->d_rcol, rcol.size() * 2));
    CR_CUDA(ctx, cudaMemcpyAsync(s->d_nbr, nbr.data(), nbr.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    CR_CUDA(ctx, cudaMemcpyAsync(s->d_rrp, rrp.data(), rrp.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    CR_CUDA(ctx, cudaMemcpyAsync(s->d_rcol, rcol.data(), rcol.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
    // uncovered-slot masks of the folded first pass (two columns, out-degrees <= 32), bit j
    // for the j-th out-neighbour of r: plane 0 [c][r] slots of r outside {c} + N(c), plane 1
    // [c][r] slots of r other than c; masks of cover_w bytes, rows padded to npad robbers
    s->cover_w = 0;
    if (s->cols == 2 && s->maxdeg <= 32) {
        const int W = s->maxdeg <= 8 ? 1 : (s->maxdeg <= 16 ? 2 : 4);
        const int n = s->n, npad = (n + 7) & ~7;
        const size_t plane = (size_t)n * npad;
        std::vector<uint32_t> m(2 * plane, 0);
        for (int r = 0; r < n; ++r) {
            const uint32_t e0 = s->h_rp[r], deg = s->h_rp[r + 1] - e0;
            const uint32_t all = deg == 32 ? 0xFFFFFFFFu : ((1u << deg) - 1u);
            for (int c = 0; c < n; ++c) m[(size_t)c * npad + r] = m[plane + (size_t)c * npad + r] = all;
            for (uint32_t j = 0; j < deg; ++j) {
                const int v = s->h_col[e0 + j];
                m[plane + (size_t)v * npad + r] &= ~(1u << j);   // slot j of r is the cop v
                m[(size_t)v * npad + r] &= ~(1u << j);           // ... and so lies in N[v]
                // slot j of r lies in N(c) for every c with v in N(c), i.e. c an in-neighbour of v
                for (uint32_t f = rrp[v]; f < rrp[v + 1]; ++f) m[(size_t)rcol[f] * npad + r] &= ~(1u << j);
            }
        }
        // plane 0 as the first pass's fast test wants it: a cop's own entry [c][c] all ones (a
        // robber on a cop is never a column-1 mark, so the entry's value is otherwise unused)
        // and the rows of cops that cannot move zero (those rows are read only when every cop
        // of the configuration can move)
        const uint32_t ones = W == 4 ? 0xFFFFFFFFu : ((1u << (8 * W)) - 1u);
        for (int c = 0; c < n; ++c) {
            m[(size_t)c * npad + c] = ones;
            if (crp[c + 1] == crp[c])
                for (int r = 0; r < npad; ++r) m[(size_t)c * npad + r] = 0u;
        }
        std::vector<uint8_t> bytes(m.size() * W);
        for (size_t i = 0; i < m.size(); ++i)
            for (int b = 0; b < W; ++b) bytes[i * W + b] = (uint8_t)(m[i] >> (8 * b));
        CR_CUDA(ctx, cudaMalloc(&s->d_cover, bytes.size()));
        CR_CUDA(ctx, cudaMemcpyAsync(s->d_cover, bytes.data(), bytes.size(), cudaMemcpyHostToDevice, ctx->stream));
        s->cover_w = W;
        s->npad = npad;
    }
    CR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CR_OK;
}

int cr_solver_create(cr_context* ctx, const cr_graph* g, int32_t k, int32_t p, int32_t rules,
                     cr_solver** out) {
    if (!ctx || !g || !out) return CR_ERR_INVALID;
    *out = nullptr;
    if (g->n <= 0) return fail(ctx, CR_ERR_INVALID, "Graph is empty or failed to load.");
    if (g->n > CR_MAX_N) return fail(ctx, CR_ERR_LIMIT, "n=%d exceeds %d vertices", g->n, CR_MAX_N);
    if (k <= 0 || k > CR_MAX_K) return fail(ctx, CR_ERR_LIMIT, "k=%d outside 1..%d", k, CR_MAX_K);
    if (p <= 0 || p > 63) return fail(ctx, CR_ERR_INVALID, "p=%d outside 1..63", p);
    const int stay = rules & (CR_COP_STAY | CR_ROBBER_STAY);
    const int base_rules = rules & ~(CR_COP_STAY | CR_ROBBER_STAY);
    if (base_rules != CR_RULES_V1 && base_rules != CR_RULES_V2) return fail(ctx, CR_ERR_INVALID, "unknown rules %d", rules);
    if (stay && base_rules != CR_RULES_V1) return fail(ctx, CR_ERR_LIMIT, "stay-allowed rules need CR_RULES_V1");
    if (!g->row_ptr || (g->row_ptr[g->n] && !g->col_idx)) return fail(ctx, CR_ERR_INVALID, "graph arrays missing");
    for (int v = 0; v < g->n; ++v)
        if (g->row_ptr[v + 1] < g->row_ptr[v]) return fail(ctx, CR_ERR_INVALID, "row_ptr not monotone");
    for (uint32_t e = 0; e < g->row_ptr[g->n]; ++e)
        if (g->col_idx[e] >= g->n) return fail(ctx, CR_ERR_INVALID, "neighbour index out of range");
    CR_CUDA(ctx, cudaSetDevice(ctx->device));

    cr_solver* s = new (std::nothrow) cr_solver();
    if (!s) return fail(ctx, CR_ERR_NOMEM, "host allocation failed");
    s->ctx = ctx;
    s->n = g->n;
    s->k = k;
    s->p = p;
    s->rules = base_rules;
    rules = base_rules;
    s->cop_stay = (stay & CR_COP_STAY) != 0;
    s->robber_stay = (stay & CR_ROBBER_STAY) != 0;
    s->S = slots_for(g->n);
    layout(s->n, k, p, rules, s->S, &s->C, &s->cols, &s->rw, &s->rwp);
    s->small = s->C * (uint64_t)s->n * s->cols < (1ull << 24);
    if (s->C == 0 || s->C >= (1ull << 32)) {
        delete s;
        return fail(ctx, CR_ERR_LIMIT, "config count C(%d,%d) outside 1..2^32-1", g->n + k - 1, k);
    }
    // the two move graphs: the input graph, plus a self-loop per vertex for a side that may stay
    auto move_graph = [&](bool self, std::vector<uint32_t>& rp, std::vector<uint16_t>& col) {
        rp.assign(1, 0);
        col.clear();
        for (int v = 0; v < g->n; ++v) {
            bool placed = !self;
            for (uint32_t e = g->row_ptr[v]; e < g->row_ptr[v + 1]; ++e) {
                if (!placed && g->col_idx[e] >= v) {
                    col.push_back((uint16_t)v);
                    placed = true;
                }
                col.push_back(g->col_idx[e]);
            }
            if (!placed) col.push_back((uint16_t)v);
            rp.push_back((uint32_t)col.size());
        }
    };
    move_graph(s->robber_stay, s->h_rp, s->h_col);
    move_graph(s->cop_stay, s->h_crp, s->h_ccol);
    for (int v = 0; v < s->n; ++v) {
        s->maxdeg = std::max<int>(s->maxdeg, s->h_rp[v + 1] - s->h_rp[v]);
        s->cop_maxdeg = std::max<int>(s->cop_maxdeg, s->h_crp[v + 1] - s->h_crp[v]);
    }
    // B[i][x] = C(n - x + k - 1 - i, k - i)
    s->h_binom.assign((size_t)k * (s->n + 1), 0);
    for (int i = 0; i < k; ++i)
        for (int x = 0; x <= s->n; ++x)
            s->h_binom[(size_t)i * (s->n + 1) + x] = (uint32_t)binom_u64((int64_t)s->n - x + k - 1 - i, k - i);

    auto bail = [&](int code) {
        free_v1(s);
        if (s->v2) crgpu::v2_destroy(s->v2);
        delete s;
        return code;
    };
#define CR_TRY(call)                                                                         \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            fail(ctx, e_ == cudaErrorMemoryAllocation ? CR_ERR_NOMEM : CR_ERR_CUDA, "%s: %s", \
                 #call, cudaGetErrorString(e_));                                             \
            return bail(e_ == cudaErrorMemoryAllocation ? CR_ERR_NOMEM : CR_ERR_CUDA);       \
        }                                                                                    \
    } while (0)
    CR_TRY(cudaMalloc(&s->d_rp, s->h_rp.size() * 4));
    CR_TRY(cudaMalloc(&s->d_col, std::max<size_t>(s->h_col.size(), 1) * 2));
    CR_TRY(cudaMalloc(&s->d_binom, s->h_binom.size() * 4));
    CR_TRY(ctx->cache.get((void**)&s->d_configs, s->C * k * 2));
    CR_TRY(cudaMalloc(&s->d_counters, 4 * sizeof(unsigned long long)));
    CR_TRY(cudaMalloc(&s->d_err, sizeof(unsigned int)));
    CR_TRY(cudaMallocHost(&s->h_pinned, (4 + kPinHist + 1) * sizeof(unsigned long long)));
    CR_TRY(cudaEventCreate(&s->ev0));
    CR_TRY(cudaEventCreate(&s->ev1));
    CR_TRY(cudaEventCreate(&s->evc0));
    CR_TRY(cudaEventCreate(&s->evc1));
    CR_TRY(cudaMemcpyAsync(s->d_rp, s->h_rp.data(), s->h_rp.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    if (!s->h_col.empty())
        CR_TRY(cudaMemcpyAsync(s->d_col, s->h_col.data(), s->h_col.size() * 2, cudaMemcpyHostToDevice, ctx->stream));
    CR_TRY(cudaMemcpyAsync(s->d_binom, s->h_binom.data(), s->h_binom.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
    CR_TRY(cudaMemsetAsync(s->d_err, 0, sizeof(unsigned int), ctx->stream));
    {
        const int grid = (int)std::min<uint64_t>((s->C + 255) / 256, (uint64_t)ctx->num_sms * 8);
        launch_unrank(s->d_binom, s->n, k, (uint32_t)s->C, s->d_configs, std::max(grid, 1), ctx->stream);
        CR_TRY(cudaGetLastError());
    }
    if (rules == CR_RULES_V1) {
        if (!pull_supported(s->S, s->rwp))
            return (fail(ctx, CR_ERR_LIMIT, "v1 rules: rows of %d vertices exceed the warp layout (n <= 512)", s->n), bail(CR_ERR_LIMIT));
        int rc = alloc_v1(s);
        if (rc) return bail(rc);
        const int per_sm = max_cop_blocks_per_sm(k, s->rwp, s->S);
        s->grid_cop = (int)std::max<uint64_t>(1, std::min<uint64_t>((s->C + 7) / 8, (uint64_t)ctx->num_sms * per_sm));
        s->grid_small = (int)std::max<uint64_t>(1, std::min<uint64_t>((s->C + 255) / 256, (uint64_t)ctx->num_sms * 4));
        if (and_smem_bytes(s->S, s->rwp, s->n) > 48 * 1024 || cop_smem_bytes(s->S, s->rwp) > 48 * 1024)
            return (fail(ctx, CR_ERR_LIMIT, "shared memory layout too large"), bail(CR_ERR_LIMIT));
    } else {
        int rc = crgpu::v2_create(&s->v2, ctx->stream, ctx->num_sms, s->n, k, p, s->d_rp, s->d_col,
                                  s->h_rp.data(), s->h_col.data(), s->d_binom, s->d_configs,
                                  (uint32_t)s->C, &ctx->err);
        if (rc) return bail(rc);
    }
    CR_TRY(cudaStreamSynchronize(ctx->stream));
#undef CR_TRY
    s->stats.slots = s->S;
    *out = s;
    return CR_OK;
}

int cr_solver_destroy(cr_solver* s) {
    if (!s) return CR_OK;
    cudaSetDevice(s->ctx->device);
    free_v1(s);
    if (s->v2) crgpu::v2_destroy(s->v2);
    delete s;
    return CR_OK;
}

static int check_err(cr_solver* s, unsigned* bits) {
    cr_context* ctx = s->ctx;
    unsigned e = 0;
    CR_CUDA(ctx, cudaMemcpyAsync(&e, s->d_err, sizeof(e), cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *bits = e;
    return CR_OK;
}

// v1 initializeCaptures on the device.
static int v1_init(cr_solver* s, uint64_t* caps) {
    cr_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    const size_t C = s->C;
    CR_CUDA(ctx, cudaEventRecord(s->ev0, st));
    CR_CUDA(ctx, cudaMemsetAsync(s->d_table, kUnmarked, C * s->n * s->cols, st));
    CR_CUDA(ctx, cudaMemsetAsync(s->d_marked, 0, (size_t)s->cols * C * s->rwp * 4, st));
    CR_CUDA(ctx, cudaMemsetAsync(s->d_fflag, 0, (size_t)s->cols * C, st));
    CR_CUDA(ctx, cudaMemsetAsync(s->d_counters, 0, 4 * sizeof(unsigned long long), st));
    CR_CUDA(ctx, cudaMemsetAsync(s->d_err, 0, sizeof(unsigned), st));
    std::vector<ColMeta> meta(s->cols);
    for (int c = 0; c < s->cols; ++c) meta[c] = ColMeta{0, kEmptyLo, -1, 0, 0, 0, 0, 0};
    // capture seeds in columns 0 and 1 (every row: the implicit list); pass 1's column-0
    // producer appends to column 0's
    meta[0] = ColMeta{0, 0, 0, 1, (int)std::min<uint64_t>(C, INT32_MAX), 0, -1, 0};
    meta[1] = ColMeta{0, 0, 0, 0, (int)std::min<uint64_t>(C, INT32_MAX), 1, -1, 0};
    CR_CUDA(ctx, cudaMemsetAsync(s->d_sync, 0, 2 * sizeof(unsigned), st));
    CR_CUDA(ctx, cudaMemcpyAsync(s->d_meta, meta.data(), sizeof(ColMeta) * s->cols, cudaMemcpyHostToDevice, st));
    V1Dev d = dev_view(s);
    launch_init(d, s->grid_small, st);
    CR_CUDA(ctx, cudaGetLastError());
    CR_CUDA(ctx, cudaEventRecord(s->ev1, st));
    CR_CUDA(ctx, cudaMemcpyAsync(s->h_pinned, s->d_counters, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    CR_CUDA(ctx, cudaStreamSynchronize(st));
    *caps = s->h_pinned[0];
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->stats.init_ms = ms;
    s->stats.kernel_launches = 1;
    return CR_OK;
}

// initializeCaptures and pass 1 of a p = 1 solve in one kernel (init_pass1_single /
// init_pass1_body): every table byte, both marked planes and both flag planes are written whole
// (column 1's frontier rows where they gained marks), so nothing is cleared first.
static int v1_init_pass1_enqueue(cr_solver* s, bool defer_list = false) {
    cr_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    CR_CUDA(ctx, cudaMemsetAsync(s->d_counters, 0, 4 * sizeof(unsigned long long), st));
    CR_CUDA(ctx, cudaMemsetAsync(s->d_err, 0, sizeof(unsigned), st));
    // column 0's frontier after pass 1 is every row (the implicit list), already consumed by
    // the fused last column, which leaves its flags clear; column 1's list is built from its
    // flags after the kernel, by k_list_compact or (defer_list) by the pass loop's entry
    ColMeta meta[2] = {ColMeta{0, 0, 0, 0, (int)std::min<uint64_t>(s->C, INT32_MAX), 0, -1, 1},
                       ColMeta{1, kEmptyLo, -1, 0, 0, 0, 0, 0, 0, defer_list ? 1 : 0}};
    CR_CUDA(ctx, cudaMemsetAsync(s->d_sync, 0, 2 * sizeof(unsigned), st));
    CR_CUDA(ctx, cudaMemcpyAsync(s->d_meta, meta, sizeof(meta), cudaMemcpyHostToDevice, st));
    V1Dev d = dev_view(s);
    CR_CUDA(ctx, cudaEventRecord(s->evc0, st));
    launch_init_pass1(d, ctx->num_sms, st);
    CR_CUDA(ctx, cudaGetLastError());
    CR_CUDA(ctx, cudaEventRecord(s->evc1, st));
    if (!defer_list) {
        launch_list_compact(d, 1, ctx->num_sms, st);   // column 1's row list, from its flags
        CR_CUDA(ctx, cudaGetLastError());
    }
    s->init_pending = false;
    s->stats.kernel_launches += defer_list ? 1 : 2;
    return CR_OK;
}

static void v1_init_pass1_time(cr_solver* s) {
    float ms = 0;
    cudaEventElapsedTime(&ms, s->evc0, s->evc1);
    s->stats.init_ms = ms;
}

static int v1_init_pass1(cr_solver* s, uint64_t* found) {
    cr_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    if (int rc = v1_init_pass1_enqueue(s)) return rc;
    CR_CUDA(ctx, cudaMemcpyAsync(s->h_pinned, s->d_counters, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    CR_CUDA(ctx, cudaStreamSynchronize(st));
    v1_init_pass1_time(s);
    *found = s->h_pinned[0];
    return CR_OK;
}

// The exact post-initializeCaptures state, for a caller that reads the table before pass 1.
static int materialize_init(cr_solver* s) {
    if (!s->init_pending) return CR_OK;
    uint64_t caps = 0;
    int rc = v1_init(s, &caps);
    if (rc) return rc;
    s->init_pending = false;
    return CR_OK;
}

// Enqueue one pass: per column a prep kernel and its producer, then the pass counter copy.
// Inside the device-side pass loop (loop set) the last column also ends the pass and runs
// column 0's prep for the next one, so the pass starts with column 0's producer; with p = 1
// the last column's prep rides on the cop turn's second launch and the last column itself.
static int v1_enqueue_pass(cr_solver* s, bool profile, bool readback = true, const LoopCtl* loop = nullptr) {
    cr_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    V1Dev d = dev_view(s);
    const bool fuse1 = loop && loop->fused_prep1;
    for (int col = 0; col < s->cols; ++col) {
        const int nx = (col + 1) % s->cols;
        if (!(loop && col == 0) && !(fuse1 && col == 1)) launch_prep(d, col, nx, s->grid_small, st);
        if (col % 2 == 0) {
            if (profile) CR_CUDA(ctx, cudaEventRecord(s->evc0, st));
            launch_cop(d, col, nx, 0, s->grid_cop, st, fuse1 && col == 0);
            if (profile) CR_CUDA(ctx, cudaEventRecord(s->evc1, st));
        } else if (col < s->cols - 1) {
            launch_cop(d, col, nx, 1, s->grid_cop, st);
        } else {
            launch_and(d, col, s->p == 1, s->grid_cop, st, loop);
        }
        CR_CUDA(ctx, cudaGetLastError());
        if (profile && col % 2 == 0) {
            // per-launch timing of the cop turn (the dominant kernel)
            CR_CUDA(ctx, cudaEventSynchronize(s->evc1));
            float ms = 0;
            cudaEventElapsedTime(&ms, s->evc0, s->evc1);
            s->stats.cop_step_ms += ms;
            s->stats.cop_step_launches += 1;
        }
    }
    if (readback)
        CR_CUDA(ctx, cudaMemcpyAsync(s->h_pinned, s->d_counters, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    return CR_OK;
}

static int v1_pass(cr_solver* s, uint64_t* found) {
    cr_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    if (ctx->profiling || s->small) {
        int rc = v1_enqueue_pass(s, ctx->profiling);
        if (rc) return rc;
    } else {
        if (!s->pass_graph) {
            cudaGraph_t graph;
            CR_CUDA(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            int rc = v1_enqueue_pass(s, false);
            cudaError_t e = cudaStreamEndCapture(st, &graph);
            if (rc) return rc;
            if (e != cudaSuccess) return fail(ctx, CR_ERR_CUDA, "pass capture: %s", cudaGetErrorString(e));
            e = cudaGraphInstantiate(&s->pass_graph, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return fail(ctx, CR_ERR_CUDA, "pass graph: %s", cudaGetErrorString(e));
        }
        CR_CUDA(ctx, cudaGraphLaunch(s->pass_graph, st));
    }
    CR_CUDA(ctx, cudaStreamSynchronize(st));
    int per_pass = s->cols;  // prep kernels
    for (int col = 0; col < s->cols; ++col)
        per_pass += col % 2 == 0 ? cop_launches_k(0, s->k, s->d_h1 != nullptr && (s->forms & CR_FORM_SEPARABLE)) : (col < s->cols - 1 ? cop_launches(1) : 1);
    s->stats.kernel_launches += per_pass;
    *found = s->h_pinned[0];
    return CR_OK;
}

int cr_solver_init(cr_solver* s, uint64_t* base_captures) {
    if (!s) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    CR_CUDA(ctx, cudaSetDevice(ctx->device));
    uint64_t caps = 0;
    s->init_pending = false;
    int rc = CR_OK;
    if (s->rules == CR_RULES_V1 && s->cols == 2 && s->S >= 2 && s->cover_w > 0 && (s->forms & CR_FORM_FUSED_FIRST)) {
        // folded into pass 1; the capture count has a closed form: every configuration
        // contributes its distinct cop vertices, and n * (multisets containing a given vertex)
        // = n * (C(n+k-1, k) - C(n+k-2, k))
        caps = (uint64_t)s->n * (binom_u64(s->n + s->k - 1, s->k) - binom_u64(s->n + s->k - 2, s->k));
        s->init_pending = true;
        s->stats.init_ms = 0;
        s->stats.kernel_launches = 0;
    } else {
        rc = s->rules == CR_RULES_V1 ? v1_init(s, &caps) : crgpu::v2_init(s->v2, &caps, &s->stats, &ctx->err);
    }
    if (rc) return rc;
    s->base_caps = caps;
    s->pass_counts.clear();
    s->initialized = true;
    s->finished = false;
    s->stats.main_ms = 0;
    s->stats.cop_step_ms = 0;
    s->stats.cop_step_launches = 0;
    s->stats.passes = 0;
    if (base_captures) *base_captures = caps;
    return CR_OK;
}

static int grow_slots_and_replay(cr_solver* s) {
    // A frontier needed more value slots than allocated: widen and replay from the start.
    cr_context* ctx = s->ctx;
    if (s->S >= 8) return fail(ctx, CR_ERR_INTERNAL, "frontier value range exceeds 8 slots");
    std::vector<uint64_t> done = s->pass_counts;
    ctx->cache.put(s->d_front);
    s->d_front = nullptr;
    ctx->cache.put(s->d_cand);
    s->d_cand = nullptr;
    ctx->cache.put(s->d_h1);
    s->d_h1 = nullptr;
    if (s->pass_graph) cudaGraphExecDestroy(s->pass_graph);
    s->pass_graph = nullptr;
    if (s->run_graph) cudaGraphExecDestroy(s->run_graph);
    s->run_graph = nullptr;
    s->S *= 2;
    if (!pull_supported(s->S, s->rwp))
        return fail(ctx, CR_ERR_LIMIT, "row too wide for %d value slots", s->S);
    CR_CUDA(ctx, ctx->cache.get((void**)&s->d_front, (size_t)s->cols * s->C * s->S * s->rwp * 4));
    CR_CUDA(ctx, ctx->cache.get((void**)&s->d_cand, (size_t)s->C * s->S * s->rwp * 4));
    CR_CUDA(ctx, cudaMemsetAsync(s->d_cand, 0, (size_t)s->C * s->S * s->rwp * 4, ctx->stream));
    CR_CUDA(ctx, cudaMemsetAsync(s->d_cbits, 0, cand_bits_bytes(s->C), ctx->stream));
    if (const uint64_t hb = h1_bytes(s->n, s->k, s->S, s->rwp)) CR_CUDA(ctx, ctx->cache.get((void**)&s->d_h1, hb));
    const int per_sm = max_cop_blocks_per_sm(s->k, s->rwp, s->S);
    s->grid_cop = (int)std::max<uint64_t>(1, std::min<uint64_t>((s->C + 7) / 8, (uint64_t)ctx->num_sms * per_sm));
    uint64_t caps;
    int rc = v1_init(s, &caps);
    if (rc) return rc;
    s->stats.slots = s->S;
    for (size_t i = 0; i < done.size(); ++i) {
        uint64_t f;
        rc = v1_pass(s, &f);
        if (rc) return rc;
        if (f != done[i]) return fail(ctx, CR_ERR_INTERNAL, "replay diverged at pass %zu", i + 1);
    }
    return CR_OK;
}

int cr_solver_pass(cr_solver* s, uint64_t* new_wins) {
    if (!s || !new_wins) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    if (!s->initialized) return fail(ctx, CR_ERR_STATE, "initializeCaptures has not run");
    if (s->finished) { *new_wins = 0; return CR_OK; }
    CR_CUDA(ctx, cudaSetDevice(ctx->device));
    uint64_t f = 0;
    if (s->rules == CR_RULES_V2) {
        int rc = crgpu::v2_pass(s->v2, &f, &s->stats, &ctx->err);
        if (rc) return rc;
    } else {
        for (int attempt = 0;; ++attempt) {
            CR_CUDA(ctx, cudaEventRecord(s->ev0, ctx->stream));
            int rc = s->init_pending ? v1_init_pass1(s, &f) : v1_pass(s, &f);
            if (rc) return rc;
            CR_CUDA(ctx, cudaEventRecord(s->ev1, ctx->stream));
            CR_CUDA(ctx, cudaEventSynchronize(s->ev1));
            float ms = 0;
            cudaEventElapsedTime(&ms, s->ev0, s->ev1);
            s->stats.main_ms += ms;
            unsigned bits = 0;
            rc = check_err(s, &bits);
            if (rc) return rc;
            if (bits & kErrRank) return fail(ctx, CR_ERR_INTERNAL, "successor rank out of range");
            if (!(bits & kErrSlot)) break;
            if (attempt > 3) return fail(ctx, CR_ERR_INTERNAL, "value slots kept overflowing");
            rc = grow_slots_and_replay(s);
            if (rc) return rc;
        }
    }
    s->pass_counts.push_back(f);
    s->stats.passes = (int)s->pass_counts.size();
    if (f == 0) s->finished = true;
    *new_wins = f;
    return CR_OK;
}

static constexpr int kHistCap = 1 << 16;   // passes one device-side loop may run

// The pass loop graph: k_loop_enter; WHILE (flag) { one pass, ending in k_and_end }, the flag
// set by k_loop_enter and then by each pass's last column.
static int build_run_graph(cr_solver* s) {
    cr_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    if (!s->d_hist) {
        CR_CUDA(ctx, cudaMalloc(&s->d_hist, sizeof(unsigned long long) * kHistCap));
        CR_CUDA(ctx, cudaMalloc(&s->d_hist_n, sizeof(int)));
    }
    cudaGraph_t g = nullptr;
    CR_CUDA(ctx, cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle loop;
    cudaError_t e = cudaGraphConditionalHandleCreate(&loop, g, 0, cudaGraphCondAssignDefault);
    const LoopCtl ctl{s->d_hist, s->d_hist_n, kHistCap, loop, s->cols == 2 ? 1 : 0};
    const V1Dev d = dev_view(s);
    // the start node sets the loop condition (and records a first pass run just before)
    cudaGraphNode_t start = nullptr;
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(st, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        launch_loop_enter(d, ctl, s->grid_small, st);
        cudaGraph_t same = nullptr;
        e = cudaStreamEndCapture(st, &same);
    }
    size_t nodes = 1;
    if (e == cudaSuccess) e = cudaGraphGetNodes(g, &start, &nodes);
    if (e == cudaSuccess && nodes != 1) e = cudaErrorInvalidValue;
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, &start, nullptr, 1, &cp);
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(st, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                            cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        int rc = v1_enqueue_pass(s, false, false, &ctl);
        cudaGraph_t body = nullptr;
        e = cudaStreamEndCapture(st, &body);
        if (rc) {
            cudaGraphDestroy(g);
            return rc;
        }
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&s->run_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        s->run_graph = nullptr;
        return fail(ctx, CR_ERR_CUDA, "pass loop graph: %s", cudaGetErrorString(e));
    }
    return CR_OK;
}

// Passes until the fixed point in one graph launch (v1, not profiling).  Returns CR_OK with
// the counts appended to pass_counts, or leaves the state for the caller's pass-by-pass loop
// when the loop stopped on an error bit or a full history.
static int v1_run_on_device(cr_solver* s) {
    cr_context* ctx = s->ctx;
    cudaStream_t st = ctx->stream;
    if (!s->run_graph) {
        int rc = build_run_graph(s);
        if (rc) return rc;
    }
    // p = 1: the fused first pass is enqueued right before the loop, whose start node records
    // its count, so the whole solve costs one host synchronisation
    const bool first = s->init_pending;
    CR_CUDA(ctx, cudaEventRecord(s->ev0, st));
    if (first) {
        if (int rc = v1_init_pass1_enqueue(s, true)) return rc;
    }
    CR_CUDA(ctx, cudaMemsetAsync(s->d_hist_n, 0, sizeof(int), st));
    if (first) CR_CUDA(ctx, cudaMemsetAsync(s->d_hist_n, 1, 1, st));   // the length 1 (low byte)
    CR_CUDA(ctx, cudaGraphLaunch(s->run_graph, st));
    CR_CUDA(ctx, cudaEventRecord(s->ev1, st));
    unsigned long long* hist_pin = s->h_pinned + 4;
    unsigned* tail = reinterpret_cast<unsigned*>(s->h_pinned + 4 + kPinHist);   // [0] length, [1] error bits
    CR_CUDA(ctx, cudaMemcpyAsync(hist_pin, s->d_hist, sizeof(unsigned long long) * kPinHist, cudaMemcpyDeviceToHost, st));
    CR_CUDA(ctx, cudaMemcpyAsync(&tail[0], s->d_hist_n, sizeof(int), cudaMemcpyDeviceToHost, st));
    CR_CUDA(ctx, cudaMemcpyAsync(&tail[1], s->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CR_CUDA(ctx, cudaStreamSynchronize(st));
    float ms = 0;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->stats.main_ms += ms;
    if (first) v1_init_pass1_time(s);
    const int n = (int)tail[0];
    const unsigned bits = tail[1];
    if (n <= 0 || n > kHistCap) return fail(ctx, CR_ERR_INTERNAL, "pass loop ran %d passes", n);
    std::vector<unsigned long long> h(hist_pin, hist_pin + std::min(n, kPinHist));
    if (n > kPinHist) {
        h.resize(n);
        CR_CUDA(ctx, cudaMemcpy(h.data() + kPinHist, s->d_hist + kPinHist, sizeof(unsigned long long) * (n - kPinHist),
                                cudaMemcpyDeviceToHost));
    }
    const int loop_passes = first ? n - 1 : n;
    // prep kernels: column 0's runs in the previous pass's last column, and with p = 1 the last
    // column's in the cop turn and the last column
    int per_pass = s->cols == 2 ? 0 : s->cols - 1;
    for (int col = 0; col < s->cols; ++col)
        per_pass += col % 2 == 0 ? cop_launches_k(0, s->k, s->d_h1 != nullptr && (s->forms & CR_FORM_SEPARABLE)) : (col < s->cols - 1 ? cop_launches(1) : 1);
    s->stats.kernel_launches += (int64_t)per_pass * loop_passes + 1;   // and the loop's entry
    if (bits & kErrRank) return fail(ctx, CR_ERR_INTERNAL, "successor rank out of range");
    if (bits & kErrSlot) {
        // the last pass overflowed its value slots: keep the passes before it, widen the slots
        // and replay them; the caller continues pass by pass
        for (int i = 0; i + 1 < n; ++i) s->pass_counts.push_back(h[i]);
        return grow_slots_and_replay(s);
    }
    for (int i = 0; i < n; ++i) s->pass_counts.push_back(h[i]);
    s->stats.passes = (int)s->pass_counts.size();
    if (h[n - 1] == 0) s->finished = true;
    return CR_OK;
}

int cr_solver_run(cr_solver* s, uint64_t* pass_counts, int32_t cap, int32_t* passes) {
    if (!s) return CR_ERR_INVALID;
    if (s->initialized && !s->finished && s->rules == CR_RULES_V1 && !s->ctx->profiling && !s->small) {
        CR_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
        int rc = v1_run_on_device(s);   // with the fused first pass when it is still pending
        if (rc) return rc;
    }
    for (int i = 0; i < 1 << 16 && !s->finished; ++i) {
        uint64_t f;
        int rc = cr_solver_pass(s, &f);
        if (rc) return rc;
        if (s->finished) break;
    }
    if (!s->finished) return fail(s->ctx, CR_ERR_BUDGET, "no fixed point after 65536 passes");
    if (passes) *passes = (int32_t)s->pass_counts.size();
    if (pass_counts)
        for (size_t i = 0; i < s->pass_counts.size() && (int32_t)i < cap; ++i) pass_counts[i] = s->pass_counts[i];
    return CR_OK;
}

int cr_solver_verdict(cr_solver* s, cr_verdict* out) {
    if (!s || !out) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    CR_CUDA(ctx, cudaSetDevice(ctx->device));
    if (int rc = materialize_init(s)) return rc;
    cudaStream_t st = ctx->stream;
    const unsigned long long init = ~0ull;
    CR_CUDA(ctx, cudaMemcpyAsync(s->d_counters + 1, &init, sizeof(init), cudaMemcpyHostToDevice, st));
    if (s->rules == CR_RULES_V1) {
        V1Dev d = dev_view(s);
        launch_verdict(d, s->cols, s->d_counters + 1, s->grid_cop, st);
    } else {
        crgpu::v2_verdict(s->v2, s->d_counters + 1);
    }
    CR_CUDA(ctx, cudaGetLastError());
    CR_CUDA(ctx, cudaMemcpyAsync(s->h_pinned + 1, s->d_counters + 1, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    CR_CUDA(ctx, cudaStreamSynchronize(st));
    const unsigned long long key = s->h_pinned[1];
    memset(out, 0, sizeof(*out));
    if (key == ~0ull || (int)(key >> 32) >= kMaxRound) {
        out->win = 0;
        out->best_config = -1;
        out->capture_plies = kMaxRound;
        return CR_OK;
    }
    out->win = 1;
    out->best_config = (int64_t)(key & 0xFFFFFFFFull);
    out->capture_plies = (int32_t)(key >> 32);
    uint16_t pos[CR_MAX_K];
    CR_CUDA(ctx, cudaMemcpyAsync(pos, s->d_configs + (size_t)out->best_config * s->k, s->k * 2, cudaMemcpyDeviceToHost, st));
    CR_CUDA(ctx, cudaStreamSynchronize(st));
    for (int i = 0; i < s->k; ++i) out->positions[i] = pos[i];
    return CR_OK;
}

int cr_solver_sizes(cr_solver* s, cr_table_sizes* out) {
    if (!s || !out) return CR_ERR_INVALID;
    out->config_count = s->C;
    out->columns = s->cols;
    out->num_states = s->C * (uint64_t)s->n * s->cols;
    out->k = s->k;
    out->n = s->n;
    out->pad = 0;
    out->transitions = s->n_trans;
    return CR_OK;
}

int cr_solver_stats(cr_solver* s, cr_solve_stats* out) {
    if (!s || !out) return CR_ERR_INVALID;
    *out = s->stats;
    uint64_t res = s->base_caps * (s->rules == CR_RULES_V1 ? 2 : 1);
    for (uint64_t c : s->pass_counts) res += c;
    out->resolved = res;
    return CR_OK;
}

int cr_solver_v2_hash_stats(cr_solver* s, cr_v2_hash_stats* out) {
    if (!s || !out) return CR_ERR_INVALID;
    *out = s->v2 ? crgpu::v2_hash_stats(s->v2) : cr_v2_hash_stats{};
    return CR_OK;
}

int cr_solver_set_forms(cr_solver* s, uint32_t mask) {
    if (!s) return CR_ERR_INVALID;
    if ((mask & ~CR_FORMS_ALL) || !(mask & (CR_FORM_PUSH | CR_FORM_PULL)))
        return fail(s->ctx, CR_ERR_INVALID, "forms: mask 0x%x (unknown bits, or neither push nor pull)", mask);
    if (s->rules != CR_RULES_V1 && mask != CR_FORMS_ALL)
        return fail(s->ctx, CR_ERR_INVALID, "forms: v2 solves have one form");
    if (mask == s->forms) return CR_OK;
    s->forms = mask;
    // the captured pass graphs hold the old device view
    if (s->pass_graph) cudaGraphExecDestroy(s->pass_graph);
    s->pass_graph = nullptr;
    if (s->run_graph) cudaGraphExecDestroy(s->run_graph);
    s->run_graph = nullptr;
    return CR_OK;
}

int cr_solver_set_v2_hash_capacity(cr_solver* s, uint64_t slots) {
    if (!s) return CR_ERR_INVALID;
    if (!s->v2) return CR_OK;   // v1 rules: no cloud table
    return crgpu::v2_set_hash_capacity(s->v2, slots, &s->ctx->err);
}

static const uint8_t* table_ptr(const cr_solver* s) {
    return s->rules == CR_RULES_V1 ? s->d_table : crgpu::v2_table(s->v2);
}

int cr_solver_digest(cr_solver* s, uint64_t* digest) {
    if (!s || !digest) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    CR_CUDA(ctx, cudaSetDevice(ctx->device));
    if (int rc = materialize_init(s)) return rc;
    cudaStream_t st = ctx->stream;
    CR_CUDA(ctx, cudaMemsetAsync(s->d_counters + 2, 0, sizeof(unsigned long long), st));
    launch_digest(table_ptr(s), s->C * (size_t)s->n * s->cols, s->d_counters + 2, ctx->num_sms * 4, st);
    CR_CUDA(ctx, cudaGetLastError());
    CR_CUDA(ctx, cudaMemcpyAsync(s->h_pinned + 2, s->d_counters + 2, 8, cudaMemcpyDeviceToHost, st));
    CR_CUDA(ctx, cudaStreamSynchronize(st));
    *digest = s->h_pinned[2];
    return CR_OK;
}

int cr_solver_device_states(cr_solver* s, void** dev_ptr, size_t* bytes) {
    if (!s || !dev_ptr || !bytes) return CR_ERR_INVALID;
    CR_CUDA(s->ctx, cudaSetDevice(s->ctx->device));
    if (int rc = materialize_init(s)) return rc;
    *dev_ptr = (void*)table_ptr(s);
    *bytes = s->C * (size_t)s->n * s->cols;
    return CR_OK;
}

int cr_solver_read_states(cr_solver* s, uint8_t* dst, size_t bytes) {
    if (!s || !dst) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    const size_t need = s->C * (size_t)s->n * s->cols;
    if (bytes < need) return fail(ctx, CR_ERR_INVALID, "states buffer holds %zu of %zu bytes", bytes, need);
    CR_CUDA(ctx, cudaSetDevice(ctx->device));
    if (int rc = materialize_init(s)) return rc;
    CR_CUDA(ctx, cudaMemcpyAsync(dst, table_ptr(s), need, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CR_OK;
}

int cr_solver_read_configs(cr_solver* s, uint8_t* dst, size_t bytes) {
    if (!s || !dst) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    if (s->n > 256) return fail(ctx, CR_ERR_LIMIT, "the table file stores vertices as uint8 (n <= 256)");
    const size_t cnt = s->C * (size_t)s->k;
    if (bytes < cnt) return fail(ctx, CR_ERR_INVALID, "configs buffer too small");
    std::vector<uint16_t> h(cnt);
    CR_CUDA(ctx, cudaMemcpyAsync(h.data(), s->d_configs, cnt * 2, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < cnt; ++i) dst[i] = (uint8_t)h[i];
    return CR_OK;
}

int cr_solver_build_transitions(cr_solver* s, uint64_t* total) {
    if (!s) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    CR_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    if (!s->d_heads) {
        const int cap = trans_cap(s->k, s->cop_maxdeg);
        if (cap > 8192) return fail(ctx, CR_ERR_LIMIT, "successor fan-out %d too large for the CSR builder", cap);
        unsigned long long* counts = nullptr;
        CR_CUDA(ctx, cudaMalloc(&counts, s->C * 8));
        CR_CUDA(ctx, cudaMalloc(&s->d_heads, (s->C + 1) * 8));
        CR_CUDA(ctx, cudaMemsetAsync(s->d_err, 0, sizeof(unsigned), st));
        const int grid = ctx->num_sms * 8;
        const uint32_t* trp = s->d_crp ? s->d_crp : s->d_rp;
        const uint16_t* tcol = s->d_ccol ? s->d_ccol : s->d_col;
        launch_trans(s->k, s->d_configs, (uint32_t)s->C, s->n, trp, tcol, s->d_binom, cap, counts,
                     nullptr, nullptr, s->d_err, grid, st);
        launch_scan(counts, s->d_heads, (uint32_t)s->C, st);
        CR_CUDA(ctx, cudaGetLastError());
        unsigned long long tot = 0;
        CR_CUDA(ctx, cudaMemcpyAsync(&tot, s->d_heads + s->C, 8, cudaMemcpyDeviceToHost, st));
        CR_CUDA(ctx, cudaStreamSynchronize(st));
        cudaFree(counts);
        s->n_trans = tot;
        CR_CUDA(ctx, cudaMalloc(&s->d_trans, std::max<uint64_t>(tot, 1) * 8));
        launch_trans(s->k, s->d_configs, (uint32_t)s->C, s->n, trp, tcol, s->d_binom, cap, nullptr,
                     s->d_heads, s->d_trans, s->d_err, grid, st);
        CR_CUDA(ctx, cudaGetLastError());
        unsigned bits = 0;
        int rc = check_err(s, &bits);
        if (rc) return rc;
        if (bits) return fail(ctx, CR_ERR_LIMIT, "successor fan-out exceeded the builder's buffer");
    }
    if (total) *total = s->n_trans;
    return CR_OK;
}

int cr_solver_perfect_game(cr_solver* s, int64_t* configs, int32_t* robbers, int32_t cap,
                           int32_t* count, int32_t* captured) {
    if (!s || !configs || !robbers || !count || !captured || cap <= 0) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    if (s->rules != CR_RULES_V1 || s->cols != 2 || s->cop_stay || s->robber_stay)
        return fail(ctx, CR_ERR_LIMIT, "the perfect game reads two-column (v1, p = 1) tables without stays");
    if (!s->finished) return fail(ctx, CR_ERR_STATE, "the solve has not reached its fixed point");
    *count = 0;
    *captured = 0;
    cr_verdict v;
    int rc = cr_solver_verdict(s, &v);
    if (rc) return rc;
    if (!v.win) return CR_OK;
    rc = cr_solver_build_transitions(s, nullptr);
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    long long* d_c = nullptr;
    int* d_r = nullptr;
    CR_CUDA(ctx, cudaMalloc(&d_c, sizeof(long long) * cap + sizeof(int) * (cap + 2)));
    d_r = reinterpret_cast<int*>(d_c + cap);
    launch_game(s->d_table, s->d_configs, s->d_heads, s->d_trans, s->d_rp, s->d_col, s->n, s->k,
                (long long)v.best_config, cap, d_c, d_r, d_r + cap, d_r + cap + 1, st);
    cudaError_t e = cudaGetLastError();
    int meta[2] = {0, 0};
    std::vector<long long> hc(cap);
    if (e == cudaSuccess) e = cudaMemcpyAsync(meta, d_r + cap, sizeof(meta), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc.data(), d_c, sizeof(long long) * cap, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(robbers, d_r, sizeof(int) * cap, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d_c);
    if (e != cudaSuccess) return fail(ctx, CR_ERR_CUDA, "perfect game: %s", cudaGetErrorString(e));
    for (int i = 0; i < meta[0] && i < cap; ++i) configs[i] = hc[i];
    *count = meta[0];
    *captured = meta[1];
    return CR_OK;
}

int cr_solver_read_transitions(cr_solver* s, uint64_t* heads, size_t heads_len, uint64_t* data,
                               size_t data_len) {
    if (!s) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    int rc = cr_solver_build_transitions(s, nullptr);
    if (rc) return rc;
    if (heads) {
        if (heads_len < s->C + 1) return fail(ctx, CR_ERR_INVALID, "heads buffer too small");
        CR_CUDA(ctx, cudaMemcpyAsync(heads, s->d_heads, (s->C + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream));
    }
    if (data) {
        if (data_len < s->n_trans) return fail(ctx, CR_ERR_INVALID, "transitions buffer too small");
        if (s->n_trans) CR_CUDA(ctx, cudaMemcpyAsync(data, s->d_trans, s->n_trans * 8, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CR_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return CR_OK;
}

int cr_solver_write_table_file(cr_solver* s, const char* path) {
    // CacheManager::saveAuxGraph (lib/include/CacheManager.h:28-75): 12 x u64 header
    // (k, N, columns, configCount, numStates, sizeof(T)=1, copSelf=0, robberSelf=0, four
    // section offsets), then configs u8, heads u64, transitions u64, states.
    if (!s || !path) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    int rc = cr_solver_build_transitions(s, nullptr);
    if (rc) return rc;
    const uint64_t cfg = s->C * (uint64_t)s->k, heads = (s->C + 1) * 8, trans = s->n_trans * 8;
    const uint64_t states = s->C * (uint64_t)s->n * s->cols;
    uint64_t hdr[12] = {(uint64_t)s->k, (uint64_t)s->n, (uint64_t)s->cols, s->C, states, 1,
                        (uint64_t)s->cop_stay, (uint64_t)s->robber_stay,
                        96, 96 + cfg, 96 + cfg + heads, 96 + cfg + heads + trans};
    FILE* f = fopen(path, "wb");
    if (!f) return fail(ctx, CR_ERR_IO, "cannot open %s for writing", path);
    std::vector<uint8_t> buf;
    bool ok = fwrite(hdr, 1, 96, f) == 96;
    buf.resize(cfg);
    rc = cr_solver_read_configs(s, buf.data(), buf.size());
    if (rc) { fclose(f); return rc; }
    ok = ok && fwrite(buf.data(), 1, cfg, f) == cfg;
    std::vector<uint64_t> hv(s->C + 1), tv(std::max<uint64_t>(s->n_trans, 1));
    rc = cr_solver_read_transitions(s, hv.data(), hv.size(), tv.data(), tv.size());
    if (rc) { fclose(f); return rc; }
    ok = ok && fwrite(hv.data(), 1, heads, f) == heads;
    ok = ok && (trans == 0 || fwrite(tv.data(), 1, trans, f) == trans);
    buf.resize(states);
    rc = cr_solver_read_states(s, buf.data(), buf.size());
    if (rc) { fclose(f); return rc; }
    ok = ok && fwrite(buf.data(), 1, states, f) == states;
    ok = (fclose(f) == 0) && ok;
    if (!ok) return fail(ctx, CR_ERR_IO, "short write to %s", path);
    return CR_OK;
}

int cr_solver_load_table_file(cr_solver* s, const char* path) {
    if (!s || !path) return CR_ERR_INVALID;
    cr_context* ctx = s->ctx;
    if (s->n > 256) return fail(ctx, CR_ERR_LIMIT, "the table file stores vertices as uint8 (n <= 256)");
    FILE* f = fopen(path, "rb");
    if (!f) return fail(ctx, CR_ERR_IO, "cannot open %s", path);
    std::vector<uint8_t> blob;
    {
        uint8_t buf[1 << 16];
        size_t got;
        while ((got = fread(buf, 1, sizeof(buf), f)) > 0) blob.insert(blob.end(), buf, buf + got);
        fclose(f);
    }
    if (blob.size() < 96) return fail(ctx, CR_ERR_IO, "%s: short header", path);
    uint64_t h[12];
    memcpy(h, blob.data(), 96);
    const uint64_t states = s->C * (uint64_t)s->n * s->cols;
    // the key fields (CacheManager.h:88-104): k, N, columns, configCount, numStates, the item
    // size and the self-edge rules
    if (h[0] != (uint64_t)s->k || h[1] != (uint64_t)s->n || h[2] != (uint64_t)s->cols || h[3] != s->C ||
        h[4] != states || h[5] != 1 || h[6] != (uint64_t)s->cop_stay || h[7] != (uint64_t)s->robber_stay)
        return fail(ctx, CR_ERR_INVALID, "%s was written for another solve", path);
    const uint64_t cfg = s->C * (uint64_t)s->k, heads = (s->C + 1) * 8;
    if (h[8] != 96 || h[9] != 96 + cfg || h[10] != h[9] + heads || h[11] < h[10] || (h[11] - h[10]) % 8 ||
        blob.size() != h[11] + states)
        return fail(ctx, CR_ERR_IO, "%s: sections do not match the header", path);
    std::vector<uint8_t> mine(cfg);
    int rc = cr_solver_read_configs(s, mine.data(), mine.size());
    if (rc) return rc;
    if (memcmp(mine.data(), blob.data() + h[8], cfg) != 0)
        return fail(ctx, CR_ERR_INVALID, "%s: configs section differs from this solver's", path);
    CR_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const uint64_t ntrans = (h[11] - h[10]) / 8;
    if (!s->d_heads) CR_CUDA(ctx, cudaMalloc(&s->d_heads, heads));
    if (s->d_trans && ntrans > s->n_trans) {
        cudaFree(s->d_trans);
        s->d_trans = nullptr;
    }
    if (!s->d_trans) CR_CUDA(ctx, cudaMalloc(&s->d_trans, std::max<uint64_t>(ntrans, 1) * 8));
    s->n_trans = ntrans;
    CR_CUDA(ctx, cudaMemcpyAsync(s->d_heads, blob.data() + h[9], heads, cudaMemcpyHostToDevice, st));
    if (ntrans) CR_CUDA(ctx, cudaMemcpyAsync(s->d_trans, blob.data() + h[10], ntrans * 8, cudaMemcpyHostToDevice, st));
    if (s->rules == CR_RULES_V2) {
        // the single-plane store of the v2 solver (k_cops_visibility_v2.cpp:170-182 loads the
        // same file layout with one column)
        if (int rc2 = crgpu::v2_load_states(s->v2, blob.data() + h[11], &ctx->err)) return rc2;
    } else {
        CR_CUDA(ctx, cudaMemcpyAsync(s->d_table, blob.data() + h[11], states, cudaMemcpyHostToDevice, st));
        launch_marks_from_table(s->d_table, (uint32_t)s->C, s->n, s->cols, s->rwp, s->d_marked, ctx->num_sms * 8, st);
        CR_CUDA(ctx, cudaGetLastError());
    }
    CR_CUDA(ctx, cudaStreamSynchronize(st));   // the host blob goes out of scope
    s->init_pending = false;
    s->initialized = true;
    s->finished = true;
    s->pass_counts.clear();
    return CR_OK;
}

int cr_solve(cr_context* ctx, const cr_graph* g, int32_t k, int32_t p, int32_t rules,
             uint8_t* states_out, size_t states_bytes, uint64_t* pass_counts, int32_t cap,
             int32_t* passes, cr_verdict* verdict, cr_solve_stats* stats) {
    cr_solver* s = nullptr;
    int rc = cr_solver_create(ctx, g, k, p, rules, &s);
    if (rc) return rc;
    rc = cr_solver_init(s, nullptr);
    if (!rc) rc = cr_solver_run(s, pass_counts, cap, passes);
    if (!rc && verdict) rc = cr_solver_verdict(s, verdict);
    if (!rc && states_out) rc = cr_solver_read_states(s, states_out, states_bytes);
    if (!rc && stats) rc = cr_solver_stats(s, stats);
    cr_solver_destroy(s);
    return rc;
}

}  // extern "C"
