/*
 * crgpu.h - C ABI of the GB300 k-cop retrograde solver (libcrgpu.so).
 *
 * The reference has no foreign-function interface: its solver path is the six-phase C++
 * contract of app/main.cpp:11-16,
 *
 *     bool loadGraphFile(const char*, int k, int p);   bool buildAuxGraph();
 *     bool initializeCaptures();   bool mainLoop();   bool findFinalResult();   bool outputData();
 *
 * implemented per solver translation unit (solvers/k_cops_visibility.cpp,
 * solvers/k_cops_visibility_v2.cpp) over lib/ (Graph, AdjacencyList, AuxGraph, CacheManager).
 * The entry points below are what that contract needs from a GPU: each one names the
 * reference routine it replaces.  A drop-in solver translation unit that maps the six phases
 * onto them ships as copsandrobbers_gb300/csrc/k_cops_gpu.cpp.
 *
 * Conventions: every function returns CR_OK (0) or a positive CR_ERR_* code and never
 * throws; cr_context_last_error() gives the message of the last failure on that context.
 * No C++ or CUDA types cross the boundary.  One context per host thread.  All pointers are
 * host pointers unless a name says "device".
 */
#ifndef CRGPU_H
#define CRGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CR_OK 0
#define CR_ERR_INVALID 1   /* bad argument or malformed graph */
#define CR_ERR_NOMEM 2     /* device memory exhausted or footprint admission refused */
#define CR_ERR_CUDA 3      /* a CUDA runtime call failed */
#define CR_ERR_LIMIT 4     /* size beyond what the library supports (n, k, config count) */
#define CR_ERR_INTERNAL 5  /* a device-side consistency check failed */
#define CR_ERR_BUDGET 6    /* the pass budget ran out before the fixed point */
#define CR_ERR_IO 7        /* file could not be read or written */
#define CR_ERR_STATE 8     /* phase called out of order */

/* Rule sets (the two live solvers of the reference). */
#define CR_RULES_V1 1 /* solvers/k_cops_visibility.cpp: 2p DP columns per cycle */
#define CR_RULES_V2 2 /* solvers/k_cops_visibility_v2.cpp: one plane, macro-turn search */
/* Flags OR-ed into CR_RULES_V1: the stay-allowed variants.  The reference's AuxGraph carries
 * them (copSelfEdges, lib/include/AuxGraph.h:38-39, 89-90, 203-205; robberSelfEdges,
 * solvers/k_cops_visibility.cpp:253-255) with both hard-coded off in its solvers; with both on
 * the game is the classical one of legacy/src/k_cops_4.cpp. */
#define CR_COP_STAY 0x10    /* a cop may stay on its vertex */
#define CR_ROBBER_STAY 0x20 /* the robber may stay on its vertex */

#define CR_MAX_K 4      /* cops per configuration handled by the device kernels */
#define CR_MAX_N 1024   /* vertices */

typedef struct cr_context cr_context;
typedef struct cr_solver cr_solver;

/* A graph as out-neighbour lists: row v holds the columns set in row v of the reference's
 * adjacency matrix, ascending (lib/src/AdjacencyList.cpp:33-76). */
typedef struct cr_graph {
    int32_t n;
    const uint32_t* row_ptr; /* n + 1 entries */
    const uint16_t* col_idx; /* row_ptr[n] entries */
} cr_graph;

/* findFinalResult (solvers/k_cops_visibility.cpp:301-354): the first configuration whose
 * column-0 row is all marked, with the strictly smallest worst case. */
typedef struct cr_verdict {
    int32_t win;             /* 1 = WIN, 0 = LOSS */
    int32_t capture_plies;   /* worst case of the best start; 127 on LOSS */
    int64_t best_config;     /* lexicographic config id, -1 on LOSS */
    uint16_t positions[CR_MAX_K];
} cr_verdict;

/* Sizes of the sections of the reference's table file (lib/include/CacheManager.h:33-46). */
typedef struct cr_table_sizes {
    uint64_t config_count;
    uint64_t num_states;       /* config_count * n * columns */
    int32_t columns;
    int32_t k;
    int32_t n;
    int32_t pad;
    uint64_t transitions;      /* entries of the successor CSR, 0 until built */
} cr_table_sizes;

/* Timing and traffic of the last solve, device-side (CUDA events on the solver's stream). */
typedef struct cr_solve_stats {
    double init_ms;            /* initializeCaptures; for p = 1 v1 solves, where it is folded
                                  into pass 1, the time of that one kernel */
    double main_ms;            /* mainLoop to the fixed point */
    double cop_step_ms;        /* sum over cop-turn kernel launches (when profiling) */
    int64_t cop_step_launches;
    int64_t kernel_launches;   /* kernels of this library launched by the solve */
    int32_t passes;
    int32_t slots;             /* value slots per frontier row that the solve used */
    uint64_t resolved;         /* marked states at the fixed point */
} cr_solve_stats;

/* ---- context ------------------------------------------------------------------------ */

/* stream: a cudaStream_t to launch on, or NULL for a stream owned by the context. */
int cr_context_create(int32_t device, void* stream, cr_context** out);
int cr_context_destroy(cr_context* ctx);
const char* cr_context_last_error(const cr_context* ctx);
/* Bytes of device memory a solve of this size holds (footprint admission). */
uint64_t cr_solver_footprint(int32_t n, int32_t k, int32_t p, int32_t rules);
/* 1 = time every cop-turn launch with CUDA events (fills cop_step_ms), 0 = off. */
int cr_context_set_profiling(cr_context* ctx, int32_t on);
/* Bytes of freed solver buffers (blocks of 1 MiB or more) the context keeps for the next solve
 * on it instead of returning them to the driver (default 4 GiB; 0 = keep none and release the
 * held ones now).  Repeated solves of similar size -- cr_solve in a loop, a solve server's
 * worker -- then allocate nothing.  No counterpart in the reference (it allocates host memory
 * per run, lib/src/Allocator.cpp). */
int cr_context_set_cache_limit(cr_context* ctx, uint64_t bytes);

/* ---- graph input (lib/src/Graph.cpp:15-79, lib/src/AdjacencyList.cpp:33-76) -------- */

/* Parse adjacency-matrix text exactly as Graph::Graph does.  Two-call sizing: with
 * row_ptr == NULL only *n and *nnz are written.  *n == 0 means the reference would reject
 * the file ("Graph is empty or failed to load"). */
int cr_graph_parse(const char* text, size_t len, int32_t* n, uint32_t* row_ptr,
                   uint16_t* col_idx, size_t col_cap, size_t* nnz);

/* ---- one solve, phase by phase --------------------------------------------------------- */

/* buildAuxGraph (k_cops_visibility.cpp:59-83 / v2:170-198; AuxGraph::constructFrom,
 * AuxGraph.h:59-79): allocate the device state store for (graph, k, p, rules) and build the
 * configuration table on the device. */
int cr_solver_create(cr_context* ctx, const cr_graph* g, int32_t k, int32_t p, int32_t rules,
                     cr_solver** out);
int cr_solver_destroy(cr_solver* s);
/* initializeCaptures (k_cops_visibility.cpp:85-127 / v2:200-224). */
int cr_solver_init(cr_solver* s, uint64_t* base_captures);
/* One pass of mainLoop (k_cops_visibility.cpp:142-296 / v2:437-562): *new_wins receives the
 * "Pass i: Found x new winning states" count.  0 means the fixed point was reached. */
int cr_solver_pass(cr_solver* s, uint64_t* new_wins);
/* mainLoop to the fixed point: pass_counts[i] for i < *passes (the final 0 included). */
int cr_solver_run(cr_solver* s, uint64_t* pass_counts, int32_t cap, int32_t* passes);
/* findFinalResult (k_cops_visibility.cpp:301-354 / v2:567-619). */
int cr_solver_verdict(cr_solver* s, cr_verdict* out);
int cr_solver_sizes(cr_solver* s, cr_table_sizes* out);
int cr_solver_stats(cr_solver* s, cr_solve_stats* out);
/* The states section of the table file (CacheManager.h:67): byte = marked | round << 1. */
int cr_solver_read_states(cr_solver* s, uint8_t* dst, size_t bytes);
/* Device pointer to the same table (valid until cr_solver_destroy). */
int cr_solver_device_states(cr_solver* s, void** dev_ptr, size_t* bytes);
/* The configs section (CacheManager.h:64): config_count * k bytes; n must be <= 256. */
int cr_solver_read_configs(cr_solver* s, uint8_t* dst, size_t bytes);
/* AuxGraph::createTransitions (AuxGraph.h:179-275) on the device: per-config successor
 * list, sorted and deduplicated, entries = next config id * n.  Fills sizes.transitions. */
int cr_solver_build_transitions(cr_solver* s, uint64_t* total);
int cr_solver_read_transitions(cr_solver* s, uint64_t* heads, size_t heads_len,
                               uint64_t* data, size_t data_len);
/* outputData (k_cops_visibility.cpp:356-373; CacheManager::saveAuxGraph, CacheManager.h:28-75):
 * write the whole table file (96-byte header, configs, heads, transitions, states). */
int cr_solver_write_table_file(cr_solver* s, const char* path);
/* CacheManager::loadAuxGraph (CacheManager.h:78-141; the v2 solver's hit at
 * k_cops_visibility_v2.cpp:170-182 reads the same layout with one column) into the device
 * store, v1 or v2 rules: a table file whose header matches this solver (k, n, columns, configs, states, self-edge flags) is
 * read back; its states section becomes the table, its heads and transitions sections the
 * successor CSR, its configs section is checked against the solver's own, and the marked
 * planes are rebuilt from the table bytes.  The loaded table answers cr_solver_verdict, the
 * reads and cr_solver_perfect_game as a solved one; cr_solver_init then resets every column,
 * as initializeCaptures does after a cache hit in the reference.  CR_ERR_IO when the file is
 * missing or short, CR_ERR_INVALID when it was written for another solve. */
int cr_solver_load_table_file(cr_solver* s, const char* path);

/* Deduplication of the robber clouds of a v2 solve with p >= 3.  The reference's
 * trajectoryDFS (solvers/k_cops_visibility_v2.cpp:243-341) walks every cop trajectory of every
 * state separately; the device inserts the depth-2 nodes (config, cloud) each pass reaches
 * into a hash table and evaluates each distinct node once.  Counts accumulate from
 * cr_solver_init. */
typedef struct cr_v2_hash_stats {
    uint64_t capacity;       /* slots of the table; 0 = no table (v1 rules or p < 3) */
    uint64_t child_visits;   /* non-terminal depth-2 children generated */
    uint64_t entries;        /* distinct (config, cloud) nodes stored, summed over fills */
    uint64_t fills;          /* table fills (one per pass, more when depth-1 nodes are chunked) */
} cr_v2_hash_stats;
int cr_solver_v2_hash_stats(cr_solver* s, cr_v2_hash_stats* out);
/* Resize the cloud table of a v2 solve with p >= 3 to `slots` (rounded up to a power of two,
 * at least 1024; 0 = no table, every depth-2 node is evaluated where it is reached).  A table
 * smaller than twice the depth-1 nodes fills once per chunk of slots / 2 nodes; nodes a full
 * table cannot take are evaluated directly, so the results never depend on the size.  The
 * default is twice the depth-1 nodes, capped at 2^24 slots.  Call between passes only. */
int cr_solver_set_v2_hash_capacity(cr_solver* s, uint64_t slots);

/* Kernel forms a v1 solve may choose from (all by default).  The forms are alternative ways to
 * compute the same pass, so the tables, pass counts and verdicts never depend on the mask; it
 * exists to test and compare each form.  No counterpart in the reference (its solver has one
 * sweep).  CR_FORM_PUSH and CR_FORM_PULL cannot both be off.  Takes effect from the next pass
 * (CR_FORM_FUSED_FIRST from the next cr_solver_init).  v2 solves accept CR_FORMS_ALL only. */
#define CR_FORM_FUSED_FIRST 0x01u  /* initializeCaptures and pass 1 in one kernel (p = 1) */
#define CR_FORM_PUSH        0x02u  /* cop turns of sparse frontiers: scatter to predecessors */
#define CR_FORM_PULL        0x04u  /* cop turns of dense frontiers: gather from successors */
#define CR_FORM_SEPARABLE   0x08u  /* the dense cop turn through pair rows (k = 3) */
#define CR_FORM_FRESH_LAST  0x10u  /* the last column from this pass's column-0 marks */
#define CR_FORMS_ALL        0x1Fu
int cr_solver_set_forms(cr_solver* s, uint32_t mask);

/* ---- whole solves ---------------------------------------------------------------------- */

/* loadGraphFile..findFinalResult in one call.  states_out (host, may be NULL) receives the
 * states section; pass_counts (may be NULL) the per-pass counts. */
int cr_solve(cr_context* ctx, const cr_graph* g, int32_t k, int32_t p, int32_t rules,
             uint8_t* states_out, size_t states_bytes, uint64_t* pass_counts, int32_t cap,
             int32_t* passes, cr_verdict* verdict, cr_solve_stats* stats);

/* ---- batches of small solves ----------------------------------------------------------- */

/* One (graph, k) solve of a batch.  The reference has no batched mode; each entry is what one
 * run of solvers/k_cops_visibility.cpp on that graph and k would report. */
typedef struct cr_batch_result {
    int32_t solved;          /* 1 = this k was solved (0: a smaller k already won) */
    int32_t status;          /* CR_OK or the device error of this solve */
    int32_t win;
    int32_t capture_plies;
    int32_t passes;          /* mainLoop passes, the final empty one included */
    int32_t pad;
    int64_t best_config;
    uint64_t base_captures;
    uint64_t states;         /* C(n+k-1, k) * n * 2p */
    uint64_t digest;         /* cr_solver_digest of the table */
    uint64_t pass_hash;      /* sum_i mix64(count_i ^ (i * 0xD1B54A32D192ED03)), i = 1.. */
} cr_batch_result;

typedef struct cr_batch_stats {
    double ms;               /* device time of the batch launch (CUDA events) */
    uint64_t states;         /* states of every solved (graph, k) */
    int32_t ctas;            /* persistent thread blocks */
    int32_t threads;         /* threads per block */
    int64_t slot_bytes;      /* device memory per block */
    double busy_frac;        /* mean over blocks of their busy time / the batch's time */
    double tail_ms;          /* batch time after the median block ran out of graphs */
} cr_batch_stats;

/* Cop numbers of many graphs (v1 rules, visibility p): for every graph, k = 1..kmax in
 * order, stopping at the first WIN, all in one persistent launch.  cop_number[g] = first
 * winning k or 0; results[g * kmax + k - 1] per solve.  threads_per_cta = 256, 512 or 1024, or
 * 0 to let an autotuner pick the launch shape (cached per device and batch shape).
 * n <= 128, kmax <= 3, p = 1. */
int cr_batch_solve(cr_context* ctx, const cr_graph* graphs, int32_t count, int32_t kmax, int32_t p,
                   int32_t threads_per_cta, int32_t* cop_number, cr_batch_result* results,
                   cr_batch_stats* stats);

/* The perfect game of a solved v1 table with two columns (p = 1), restating the reference's
 * util/perfect_game_extractor.py:67-171 on the device: from findFinalResult's configuration and
 * the robber vertex with the largest column-0 round, the cops take the first successor that
 * lands on the robber, else the first successor with the smallest marked column-1 round; the
 * robber takes the first neighbour with the largest marked column-0 round; until capture.
 * configs[i] / robbers[i] = the position after ply i (index 0 = the start), at most cap of
 * them; *count = positions written; *captured = 1 when the walk ended in a capture.  A LOSS
 * verdict gives *count = 0.  Needs the fixed point (CR_ERR_STATE before it). */
int cr_solver_perfect_game(cr_solver* s, int64_t* configs, int32_t* robbers, int32_t cap,
                           int32_t* count, int32_t* captured);

/* 64-bit digest of a solver's states table: sum over its 8-byte little-endian words w_j
 * (zero-padded) of mix64(w_j ^ (j * 0x9E3779B97F4A7C15)) modulo 2^64, mix64 being the
 * splitmix64 finaliser.  Used to compare batched and single solves without copying tables. */
int cr_solver_digest(cr_solver* s, uint64_t* digest);

/* ---- solve server ---------------------------------------------------------------------- */

/* A long-running solve service (the reference has no counterpart: it answers one solve per
 * process run).  Requests queue as they arrive; worker threads, each with its own stream,
 * start the first queued request whose device footprint (cr_solver_footprint) fits in the
 * memory budget left, so requests arriving while others run are admitted as soon as a worker
 * and memory free up and their solves overlap on the GPU.  Finished tables stay resident
 * until cr_server_release.  A queued request waiting more than 2 s is not overtaken. */
typedef struct cr_server cr_server;

typedef struct cr_request_result {
    int32_t status;          /* CR_OK or the solve's error code */
    int32_t win;
    int32_t capture_plies;
    int32_t passes;
    int64_t best_config;
    uint64_t base_captures;
    uint64_t states;
    uint64_t digest;         /* cr_solver_digest of the table */
    uint64_t pass_hash;      /* as in cr_batch_result */
    double queue_ms;         /* submit -> start */
    double run_ms;           /* start -> done */
    double latency_ms;       /* submit -> done */
} cr_request_result;

typedef struct cr_server_report {
    uint64_t completed, failed, queued, running, max_running;
    uint64_t memory_budget, memory_in_use, peak_memory_in_use;
    uint64_t states_done;
    double busy_ms;          /* first submit -> last completion */
} cr_server_report;

/* memory_budget = 0: 80% of the device memory free at creation. */
int cr_server_create(int32_t device, uint64_t memory_budget, int32_t workers, cr_server** out);
/* Copies the graph; CR_ERR_NOMEM if the request could never fit the budget. */
int cr_server_submit(cr_server* srv, const cr_graph* g, int32_t k, int32_t p, int32_t rules,
                     uint64_t* request_id);
/* wait_ms: 0 = do not wait, < 0 = wait until done.  CR_ERR_STATE while queued or running. */
int cr_server_poll(cr_server* srv, uint64_t request_id, int32_t wait_ms, cr_request_result* out);
int cr_server_read_states(cr_server* srv, uint64_t request_id, uint8_t* dst, size_t bytes);
/* Frees a finished request's resident table and returns its memory to the budget. */
int cr_server_release(cr_server* srv, uint64_t request_id);
int cr_server_stats(cr_server* srv, cr_server_report* out);
const char* cr_server_last_error(const cr_server* srv);
int cr_server_destroy(cr_server* srv);

/* ---- allocation-free solve ------------------------------------------------------------ */

/* No counterpart in the reference.  The v1 solve (loadGraphFile..mainLoop) for callers that
 * cannot allocate memory -- a caller working inside a memory pool or budget it does not own,
 * one that must not take the CUDA allocator's locks on its critical path, or an embedder that
 * forbids libraries from owning device memory.  The caller passes the graph as host arrays
 * and the states table as device memory it owns (states_bytes >= C(n+k-1,k) * n * 2p); all
 * other working memory is one fixed 64 MiB __device__ array inside the library, so nothing is
 * allocated: no cudaMalloc/cudaFree, no pinned host memory, no streams, events or graphs.
 *   - Limit: n <= 512 and a working set (everything but the table) within 64 MiB, e.g.
 *     n=128 with k=3 at p=1; larger solves return CR_ERR_LIMIT with the bytes needed in err.
 *   - Every GPU that loads the library holds the 64 MiB until the process exits.
 *   - The first call on a device looks up the array's device address (once per device);
 *     make it before any stream capture on that device.  The address is kept for the life of
 *     the process: after a cudaDeviceReset (or anything else that destroys the device's
 *     primary context) it is stale, so do not call this entry point again in that process.
 *   - It runs the general forms only -- initializeCaptures unfused from pass 1 and the
 *     tuple-gathering cop turn -- because the fused first pass's tables and the separable
 *     turn's pair rows need memory beyond the area; it is slower than cr_solve.
 *   - All calls share the array and leave their contents in it; each call clears what must
 *     start at zero.  Calls whose GPU work overlaps (other streams or host threads) race.
 * stream: cudaStream_t or NULL.  pass_counts[0 .. *passes) receive the per-pass counts;
 * err (may be NULL) receives a message on failure. */
int cr_solve_v1_noalloc(const cr_graph* g, int32_t k, int32_t p, void* stream,
                        uint8_t* states_dev, size_t states_bytes, uint64_t* pass_counts,
                        int32_t cap, int32_t* passes, uint64_t* base_captures, char* err,
                        size_t err_len);

#ifdef __cplusplus
}
#endif
#endif /* CRGPU_H */
