/*
 * cr_oracle.c - CPU restatement of the reference k-cop solvers.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the GPU solver is compared with: the tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it.  No product code links it,
 * and the product never falls back to it.
 *
 * It restates, for any vertex count (vertices are uint16 here, where the reference stores
 * uint8 with 255 as a terminator and so stops at 255 vertices):
 *   - cop-configuration enumeration in lexicographic order   (lib/include/AuxGraph.h:117-177)
 *   - the per-config successor CSR, sorted and deduplicated   (lib/include/AuxGraph.h:179-275)
 *   - v1 initializeCaptures + mainLoop, the 2p-column sweep    (solvers/k_cops_visibility.cpp:85-299)
 *   - v2 initializeCaptures + the snapshot macro-turn search  (solvers/k_cops_visibility_v2.cpp:200-565)
 *   - the verdict scan shared by both                          (solvers/k_cops_visibility.cpp:301-354)
 *
 * Within one v1 column every state reads only the next column, so a column's configs are
 * split across threads with results identical to the reference's serial sweep.  v2 passes
 * read a start-of-pass snapshot and buffer their marks, so its states split the same way.
 * The v2 restatement takes the exact minimum over cop trajectories directly; the reference's
 * branch-and-bound ordering and its two skip filters only prune work and do not change the
 * minimum (its file header, lines 42-55).
 *
 * Table byte = marked | (markedRound << 1); an unmarked cell holds 0xFE (markedRound = 127),
 * matching the DataItem bitfield of solvers/k_cops_visibility.cpp:20-26 on GCC.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_UNMARKED 0xFEu
#define OR_MAX_ROUND 127
#define OR_MAX_K 16
#define OR_MAX_WORDS 16 /* v2 cloud masks: up to 1024 vertices */

/* ---------------------------------------------------------------- graph helpers --- */

typedef struct {
    int n;
    const uint32_t* row_ptr; /* n + 1 */
    const uint16_t* col;     /* neighbours of v, ascending (AdjacencyList.cpp:58-68) */
} or_graph;

static int deg_of(const or_graph* g, int v) { return (int)(g->row_ptr[v + 1] - g->row_ptr[v]); }

/* ---------------------------------------------------------------- configurations --- */

/* Number of sorted k-multisets of n vertices, C(n+k-1, k), computed as AuxGraph.h:124-138. */
uint64_t or_config_count(int n, int k) {
    if (k <= 0 || n <= 0) return 0;
    int64_t n_val = n + k - 1, k_val = k;
    if (k_val > n_val) return 0;
    if (k_val == n_val) return 1;
    if (k_val > n_val / 2) k_val = n_val - k_val;
    uint64_t res = 1;
    for (int64_t i = 1; i <= k_val; ++i) res = res * (uint64_t)(n_val - i + 1) / (uint64_t)i;
    return res;
}

/* Lexicographic odometer over non-decreasing tuples (AuxGraph.h:160-176). */
void or_configs(int n, int k, uint16_t* out) {
    uint16_t cur[OR_MAX_K];
    memset(cur, 0, sizeof(cur));
    size_t off = 0;
    for (;;) {
        memcpy(out + off, cur, (size_t)k * sizeof(uint16_t));
        off += (size_t)k;
        int p = k - 1;
        while (p >= 0 && cur[p] == n - 1) p--;
        if (p < 0) break;
        cur[p]++;
        for (int i = p + 1; i < k; ++i) cur[i] = cur[p];
    }
}

static int cmp_u16(const void* a, const void* b) {
    return (int)*(const uint16_t*)a - (int)*(const uint16_t*)b;
}
static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

/* Binary search of a sorted tuple in the lexicographic config list (AuxGraph.h:223-239). */
static uint64_t find_config(const uint16_t* configs, uint64_t count, int k, const uint16_t* t) {
    uint64_t lo = 0, hi = count;
    while (lo < hi) {
        uint64_t mid = lo + (hi - lo) / 2;
        int c = 0;
        for (int i = 0; i < k && !c; ++i) c = (int)configs[mid * k + i] - (int)t[i];
        if (c == 0) return mid;
        if (c < 0) lo = mid + 1; else hi = mid;
    }
    return UINT64_MAX;
}

/* Successor list of one config: odometer over each cop's options (optionally its own vertex
 * first), sort the moved tuple, look up its id, store id * n; then sort and deduplicate
 * (AuxGraph.h:194-259).  Returns the count written to out (capacity >= prod of options). */
static size_t successors(const or_graph* g, const uint16_t* configs, uint64_t count, int k,
                         uint64_t cid, int cop_stay, uint64_t* out) {
    const uint16_t* cops = configs + cid * k;
    int optc[OR_MAX_K], odo[OR_MAX_K];
    uint16_t opt[OR_MAX_K][1025];
    for (int i = 0; i < k; ++i) {
        int c = 0;
        if (cop_stay) opt[i][c++] = cops[i];
        for (uint32_t e = g->row_ptr[cops[i]]; e < g->row_ptr[cops[i] + 1]; ++e) opt[i][c++] = g->col[e];
        optc[i] = c;
        odo[i] = 0;
    }
    size_t m = 0;
    for (int i = 0; i < k; ++i) if (optc[i] == 0) return 0;
    for (;;) {
        uint16_t t[OR_MAX_K];
        for (int i = 0; i < k; ++i) t[i] = opt[i][odo[i]];
        qsort(t, (size_t)k, sizeof(uint16_t), cmp_u16);
        uint64_t id = find_config(configs, count, k, t);
        out[m++] = id * (uint64_t)g->n;
        int p = k - 1;
        while (p >= 0) {
            if (++odo[p] < optc[p]) break;
            odo[p] = 0;
            p--;
        }
        if (p < 0) break;
    }
    qsort(out, m, sizeof(uint64_t), cmp_u64);
    size_t u = 0;
    for (size_t i = 0; i < m; ++i) if (u == 0 || out[u - 1] != out[i]) out[u++] = out[i];
    return u;
}

static size_t max_fanout(const or_graph* g, int k, int cop_stay) {
    int md = 0;
    for (int v = 0; v < g->n; ++v) if (deg_of(g, v) > md) md = deg_of(g, v);
    size_t f = 1;
    for (int i = 0; i < k; ++i) f *= (size_t)(md + (cop_stay ? 1 : 0));
    return f ? f : 1;
}

/* Transition CSR: heads[count + 1] and, when data != NULL, data[heads[count]].
 * Call once with data == NULL to size it.  Configs are independent, so both calls split them
 * across threads; the result is identical to the serial build. */
int or_transitions(int n, const uint32_t* row_ptr, const uint16_t* col, int k, int cop_stay,
                   const uint16_t* configs, uint64_t count, uint64_t* heads, uint64_t* data) {
    or_graph g = {n, row_ptr, col};
    size_t cap = max_fanout(&g, k, cop_stay);
    int fail = 0;
    if (!data) {
        heads[0] = 0;
        #pragma omp parallel reduction(| : fail)
        {
            uint64_t* buf = (uint64_t*)malloc(cap * sizeof(uint64_t));
            if (!buf) fail = 1;
            #pragma omp for schedule(dynamic, 256)
            for (int64_t c = 0; c < (int64_t)count; ++c)
                heads[c + 1] = buf ? successors(&g, configs, count, k, (uint64_t)c, cop_stay, buf) : 0;
            free(buf);
        }
        for (uint64_t c = 0; c < count; ++c) heads[c + 1] += heads[c];
        return fail;
    }
    #pragma omp parallel reduction(| : fail)
    {
        uint64_t* buf = (uint64_t*)malloc(cap * sizeof(uint64_t));
        if (!buf) fail = 1;
        #pragma omp for schedule(dynamic, 256)
        for (int64_t c = 0; c < (int64_t)count; ++c) {
            if (!buf) continue;
            size_t m = successors(&g, configs, count, k, (uint64_t)c, cop_stay, buf);
            memcpy(data + heads[c], buf, m * sizeof(uint64_t));
        }
        free(buf);
    }
    return fail;
}

/* Exact-p-hop reachability from r (k_cops_visibility.cpp:245-262), as a byte mask. */
static void hop_set(const or_graph* g, int r, int depth, int robber_stay, uint8_t* cur, uint8_t* nxt) {
    memset(cur, 0, (size_t)g->n);
    cur[r] = 1;
    for (int s = 0; s < depth; ++s) {
        memset(nxt, 0, (size_t)g->n);
        for (int v = 0; v < g->n; ++v) {
            if (!cur[v]) continue;
            if (robber_stay) nxt[v] = 1;
            for (uint32_t e = g->row_ptr[v]; e < g->row_ptr[v + 1]; ++e) nxt[g->col[e]] = 1;
        }
        memcpy(cur, nxt, (size_t)g->n);
    }
}

/* ------------------------------------------------------------------------- v1 --- */

/* One column of the v1 sweep over configs [c0, c1) (k_cops_visibility.cpp:146-290).
 * Returns the number of states marked. */
static uint64_t v1_column(const or_graph* g, int cols, int cl, const uint64_t* heads,
                          const uint64_t* trans, const uint8_t* hops, uint8_t* states,
                          int64_t c0, int64_t c1) {
    const int n = g->n;
    const int nx = (cl + 1) % cols;
    uint64_t fc = 0;
    if (cl % 2 == 0) {
        /* cop turn: OR over transitions, min + 1 (k_cops_visibility.cpp:160-197) */
        #pragma omp parallel for schedule(dynamic, 64) reduction(+ : fc)
        for (int64_t c = c0; c < c1; ++c) {
            for (int r = 0; r < n; ++r) {
                uint8_t* s = states + ((size_t)c * n + r) * cols + cl;
                if (*s & 1) continue;
                int mn = OR_MAX_ROUND, win = 0;
                for (uint64_t i = heads[c]; i < heads[c + 1]; ++i) {
                    uint8_t v = states[(trans[i] + (uint64_t)r) * cols + nx];
                    if (v & 1) { win = 1; if ((v >> 1) < mn) mn = v >> 1; }
                }
                if (win && mn + 1 < OR_MAX_ROUND) { *s = (uint8_t)(1 | ((mn + 1) << 1)); fc++; }
            }
        }
    } else if (cl < cols - 1) {
        /* deferred robber turn: direct copy + 1 (k_cops_visibility.cpp:209-228) */
        #pragma omp parallel for schedule(dynamic, 64) reduction(+ : fc)
        for (int64_t c = c0; c < c1; ++c) {
            for (int r = 0; r < n; ++r) {
                uint8_t* s = states + ((size_t)c * n + r) * cols + cl;
                if (*s & 1) continue;
                uint8_t v = states[((size_t)c * n + r) * cols + nx];
                if ((v & 1) && (v >> 1) + 1 < OR_MAX_ROUND) { *s = (uint8_t)(1 | (((v >> 1) + 1) << 1)); fc++; }
            }
        }
    } else {
        /* max col: AND over the exact-p-hop cloud, max + 1 (k_cops_visibility.cpp:235-288) */
        #pragma omp parallel for schedule(dynamic, 64) reduction(+ : fc)
        for (int64_t c = c0; c < c1; ++c) {
            for (int r = 0; r < n; ++r) {
                uint8_t* s = states + ((size_t)c * n + r) * cols + cl;
                if (*s & 1) continue;
                const uint8_t* hv = hops + (size_t)r * n;
                int all = 1, mx = 0;
                for (int v = 0; v < n; ++v) {
                    if (!hv[v]) continue;
                    uint8_t x = states[((size_t)c * n + v) * cols + nx];
                    if (!(x & 1)) { all = 0; break; }
                    if ((x >> 1) > mx) mx = x >> 1;
                }
                if (all && mx + 1 < OR_MAX_ROUND) { *s = (uint8_t)(1 | ((mx + 1) << 1)); fc++; }
            }
        }
    }
    return fc;
}

static uint8_t* v1_hops(const or_graph* g, int p, int robber_stay) {
    const int n = g->n;
    uint8_t* hops = (uint8_t*)malloc((size_t)n * n);
    uint8_t* t0 = (uint8_t*)malloc((size_t)n);
    uint8_t* t1 = (uint8_t*)malloc((size_t)n);
    if (!hops || !t0 || !t1) { free(hops); free(t0); free(t1); return NULL; }
    for (int r = 0; r < n; ++r) {
        hop_set(g, r, p, robber_stay, t0, t1);
        memcpy(hops + (size_t)r * n, t0, (size_t)n);
    }
    free(t0); free(t1);
    return hops;
}

/* initializeCaptures (k_cops_visibility.cpp:85-127). */
uint64_t or_v1_init(int n, int k, int p, const uint16_t* configs, uint64_t count, uint8_t* states) {
    const int cols = 2 * p;
    uint64_t caps = 0;
    for (uint64_t c = 0; c < count; ++c) {
        const uint16_t* cops = configs + c * k;
        for (int r = 0; r < n; ++r) {
            uint8_t* s = states + ((size_t)c * n + r) * cols;
            memset(s, OR_UNMARKED, (size_t)cols);
            int catch_ = 0;
            for (int i = 0; i < k; ++i) if (cops[i] == r) catch_ = 1;
            if (catch_) { s[0] = 1; s[1] = 1; caps++; }
        }
    }
    return caps;
}

/*
 * v1 solve.  states[(cid * n + r) * cols + col], cols = 2p.  pass_counts receives the
 * "Pass i: Found x new winning states" numbers (the final zero included); returns the pass
 * count, or -1 on allocation failure / -2 when max_passes is too small.
 * cop_stay / robber_stay select the self-edge rules (hard-coded FALSE in the reference,
 * k_cops_visibility.cpp:63-64).
 */
int or_v1_solve(int n, const uint32_t* row_ptr, const uint16_t* col, int k, int p,
                int cop_stay, int robber_stay, const uint16_t* configs, uint64_t count,
                const uint64_t* heads, const uint64_t* trans, uint8_t* states,
                uint64_t* base_captures, uint64_t* pass_counts, int max_passes, int threads) {
    or_graph g = {n, row_ptr, col};
    const int cols = 2 * p;
    (void)cop_stay; /* carried by the transition CSR passed in */
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    *base_captures = or_v1_init(n, k, p, configs, count, states);
    uint8_t* hops = v1_hops(&g, p, robber_stay);
    if (!hops) return -1;
    int passes = 0;
    for (;;) {
        if (passes >= max_passes) { free(hops); return -2; }
        uint64_t found = 0;
        for (int cl = 0; cl < cols; ++cl)
            found += v1_column(&g, cols, cl, heads, trans, hops, states, 0, (int64_t)count);
        pass_counts[passes++] = found;
        if (found == 0) break;
    }
    free(hops);
    return passes;
}

/* CPU-baseline sample: the columns of one v1 pass restricted to configs [c0, c1), on a table
 * prepared by or_v1_init.  Returns the states marked. */
uint64_t or_v1_sweep_slice(int n, const uint32_t* row_ptr, const uint16_t* col, int k, int p,
                           const uint64_t* heads, const uint64_t* trans, uint8_t* states,
                           int64_t c0, int64_t c1, int threads) {
    or_graph g = {n, row_ptr, col};
    (void)k;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    uint8_t* hops = v1_hops(&g, p, 0);
    if (!hops) return 0;
    uint64_t found = 0;
    for (int cl = 0; cl < 2 * p; ++cl) found += v1_column(&g, 2 * p, cl, heads, trans, hops, states, c0, c1);
    free(hops);
    return found;
}

/* Verdict scan over column 0 (k_cops_visibility.cpp:301-331): the first config whose every
 * robber position is marked, with the strictly smallest worst case.  Returns the config id
 * or -1; *worst receives the capture time in plies. */
int64_t or_verdict(int n, uint64_t count, int cols, const uint8_t* states, int* worst) {
    int64_t best = -1;
    int overall = OR_MAX_ROUND;
    for (uint64_t c = 0; c < count; ++c) {
        int all = 1, wc = 0;
        for (int r = 0; r < n; ++r) {
            uint8_t s = states[((size_t)c * n + r) * cols];
            if (!(s & 1)) { all = 0; break; }
            if ((s >> 1) > wc) wc = s >> 1;
        }
        if (all && wc < overall) { overall = wc; best = (int64_t)c; }
    }
    *worst = overall;
    return best;
}

/* ------------------------------------------------------------------------- v2 --- */

typedef struct { uint64_t w[OR_MAX_WORDS]; } vmask;

typedef struct {
    const or_graph* g;
    int k, p, words;
    const uint64_t* heads;
    const uint64_t* trans;
    const vmask* nbr;
    const vmask* copm;
    const vmask* marked; /* start-of-pass snapshot */
    const uint8_t* states;
} v2ctx;

static int vm_empty(const vmask* m, int w) {
    uint64_t x = 0;
    for (int i = 0; i < w; ++i) x |= m->w[i];
    return x == 0;
}

/* Minimum ply cost over all cop trajectories from (cid_prev, cloud) at step d
 * (solvers/k_cops_visibility_v2.cpp:243-341): a cop ply that empties the cloud costs 2d-1,
 * a robber ply that empties it costs 2d, and at d == p a boundary whose every cloud vertex is
 * marked in the snapshot costs 2p + max markedRound.  INT_MAX = no winning trajectory. */
static int v2_eval(const v2ctx* x, int d, uint64_t cid_prev, const vmask* cloud) {
    const int n = x->g->n, w = x->words;
    int best = INT_MAX;
    for (uint64_t i = x->heads[cid_prev]; i < x->heads[cid_prev + 1]; ++i) {
        uint64_t cn = x->trans[i] / (uint64_t)n;
        const vmask* occ = &x->copm[cn];
        vmask mid;
        for (int j = 0; j < w; ++j) mid.w[j] = cloud->w[j] & ~occ->w[j];
        if (vm_empty(&mid, w)) return 2 * d - 1; /* floor for this depth */
        vmask nxt;
        memset(&nxt, 0, sizeof(nxt));
        for (int j = 0; j < w; ++j) {
            uint64_t b = mid.w[j];
            while (b) {
                int v = j * 64 + __builtin_ctzll(b);
                b &= b - 1;
                for (int q = 0; q < w; ++q) nxt.w[q] |= x->nbr[v].w[q];
            }
        }
        for (int j = 0; j < w; ++j) nxt.w[j] &= ~occ->w[j];
        if (vm_empty(&nxt, w)) { if (2 * d < best) best = 2 * d; continue; }
        if (d == x->p) {
            const vmask* mk = &x->marked[cn];
            int sub = 1;
            for (int j = 0; j < w; ++j) if (nxt.w[j] & ~mk->w[j]) sub = 0;
            if (!sub) continue;
            int mx = 0;
            for (int j = 0; j < w; ++j) {
                uint64_t b = nxt.w[j];
                while (b) {
                    int v = j * 64 + __builtin_ctzll(b);
                    b &= b - 1;
                    int rd = x->states[cn * (uint64_t)n + (uint64_t)v] >> 1;
                    if (rd > mx) mx = rd;
                }
            }
            int cost = 2 * x->p + mx;
            if (cost < best) best = cost;
        } else {
            if (2 * d + 1 >= best) continue; /* deeper outcomes cost at least 2(d+1)-1 */
            int sub = v2_eval(x, d + 1, cn, &nxt);
            if (sub < best) best = sub;
        }
    }
    return best;
}

/* v2 solve over a single plane states[cid * n + r] (solvers/k_cops_visibility_v2.cpp:200-565).
 * Returns the number of passes, -1 on allocation failure, -2 if max_passes is too small,
 * -3 if n exceeds the mask width. */
int or_v2_solve(int n, const uint32_t* row_ptr, const uint16_t* col, int k, int p,
                const uint16_t* configs, uint64_t count, const uint64_t* heads,
                const uint64_t* trans, uint8_t* states, uint64_t* base_captures,
                uint64_t* pass_counts, int max_passes, int threads) {
    or_graph g = {n, row_ptr, col};
    if (n > OR_MAX_WORDS * 64) return -3;
    const int words = (n + 63) / 64;
    (void)threads;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    uint64_t caps = 0;
    for (uint64_t c = 0; c < count; ++c) {
        const uint16_t* cops = configs + c * k;
        for (int r = 0; r < n; ++r) {
            int catch_ = 0;
            for (int i = 0; i < k; ++i) if (cops[i] == r) catch_ = 1;
            states[c * (uint64_t)n + r] = catch_ ? 1 : OR_UNMARKED;
            caps += (uint64_t)catch_;
        }
    }
    *base_captures = caps;

    vmask* nbr = (vmask*)calloc((size_t)n, sizeof(vmask));
    vmask* copm = (vmask*)calloc((size_t)count, sizeof(vmask));
    vmask* marked = (vmask*)calloc((size_t)count, sizeof(vmask));
    uint8_t* cost = (uint8_t*)malloc((size_t)count * n);
    if (!nbr || !copm || !marked || !cost) { free(nbr); free(copm); free(marked); free(cost); return -1; }
    for (int v = 0; v < n; ++v)
        for (uint32_t e = row_ptr[v]; e < row_ptr[v + 1]; ++e) nbr[v].w[col[e] >> 6] |= 1ull << (col[e] & 63);
    for (uint64_t c = 0; c < count; ++c)
        for (int i = 0; i < k; ++i) copm[c].w[configs[c * k + i] >> 6] |= 1ull << (configs[c * k + i] & 63);

    v2ctx x = {&g, k, p, words, heads, trans, nbr, copm, marked, states};
    int passes = 0;
    for (;;) {
        if (passes >= max_passes) { free(nbr); free(copm); free(marked); free(cost); return -2; }
        for (uint64_t c = 0; c < count; ++c) {
            memset(&marked[c], 0, sizeof(vmask));
            for (int r = 0; r < n; ++r)
                if (states[c * (uint64_t)n + r] & 1) marked[c].w[r >> 6] |= 1ull << (r & 63);
        }
        uint64_t found = 0;
        #pragma omp parallel for schedule(dynamic, 1) reduction(+ : found)
        for (int64_t c = 0; c < (int64_t)count; ++c) {
            for (int r = 0; r < n; ++r) {
                uint8_t* out = &cost[(size_t)c * n + r];
                *out = 0xFF;
                if (states[(size_t)c * n + r] & 1) continue;
                vmask start;
                memset(&start, 0, sizeof(start));
                start.w[r >> 6] = 1ull << (r & 63);
                int b = v2_eval(&x, 1, (uint64_t)c, &start);
                if (b < OR_MAX_ROUND) { *out = (uint8_t)b; found++; }
            }
        }
        for (size_t i = 0; i < (size_t)count * n; ++i)
            if (cost[i] != 0xFF) states[i] = (uint8_t)(1 | (cost[i] << 1));
        pass_counts[passes++] = found;
        if (found == 0) break;
    }
    free(nbr); free(copm); free(marked); free(cost);
    return passes;
}
