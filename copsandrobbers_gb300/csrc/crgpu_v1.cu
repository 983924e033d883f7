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
#include "crgpu_internal.cuh"

namespace crgpu {

#define FULL_MASK 0xFFFFFFFFu

template <int VW> struct Vec;
template <> struct Vec<1> {
    uint32_t v[1];
    __device__ void zero() { v[0] = 0; }
    __device__ void load_or(const uint32_t* p) { v[0] |= __ldg(p); }
};
template <> struct Vec<2> {
    uint32_t v[2];
    __device__ void zero() { v[0] = v[1] = 0; }
    __device__ void load_or(const uint32_t* p) {
        uint2 x = __ldg(reinterpret_cast<const uint2*>(p));
        v[0] |= x.x; v[1] |= x.y;
    }
};
template <> struct Vec<4> {
    uint32_t v[4];
    __device__ void zero() { v[0] = v[1] = v[2] = v[3] = 0; }
    __device__ void load_or(const uint32_t* p) {
        uint4 x = __ldg(reinterpret_cast<const uint4*>(p));
        v[0] |= x.x; v[1] |= x.y; v[2] |= x.z; v[3] |= x.w;
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
        }
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
// frontiers of columns 0 and 1 (value 0, slot 0).
__global__ void k_init(V1Dev d, int K) {
    unsigned long long caps = 0;
    const int n = d.g.n, rwp = d.g.rwp, S = d.S;
    for (uint32_t cid = blockIdx.x * blockDim.x + threadIdx.x; cid < d.C;
         cid += gridDim.x * blockDim.x) {
        const uint16_t* cc = d.configs + (size_t)cid * K;
        int prev = -1;
        for (int i = 0; i < K; ++i) {
            int r = cc[i];
            if (r == prev) continue;
            prev = r;
            caps++;
            size_t cell = ((size_t)cid * n + r) * d.cols;
            d.table[cell] = 1;
            d.table[cell + 1] = 1;
            uint32_t bit = 1u << (r & 31);
            int w = r >> 5;
            for (int c = 0; c < 2; ++c) {
                d.marked[((size_t)c * d.C + cid) * rwp + w] |= bit;
                d.front[(((size_t)c * d.C + cid) * S) * rwp + w] |= bit;
            }
        }
        d.fflag[cid] = 1;
        d.fflag[(size_t)d.C + cid] = 1;
    }
    caps = __reduce_add_sync(FULL_MASK, (unsigned)caps);
    if ((threadIdx.x & 31) == 0 && caps) atomicAdd(d.pass_new, caps);
}

// Cop turn (direct == 0) or deferred robber turn (direct == 1) into column `col` from the
// frontier of column nx.  One warp per configuration row; lanes split each successor row
// (S_used slots * rwp words) into VW-word chunks, L lanes per successor, 32/L successors at a
// time, and OR the chunks of every successor whose frontier row is non-empty.
template <int K, int VW>
__global__ void __launch_bounds__(256) k_cop(V1Dev d, int col, int nx, int direct) {
    extern __shared__ uint32_t sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = d.g.n, rw = d.g.rw, rwp = d.g.rwp, S = d.S;
    const ColMeta mi = d.meta[nx];
    if (mi.hi < mi.lo) return;  // empty input frontier: nothing can change
    const int base_in = mi.base;
    const int s_used = min(mi.hi - base_in + 1, S);
    const int out_base = d.meta[col].base;
    const int append = d.meta[col].append;
    const int CH = s_used * rwp / VW;
    int L = 1;
    while (L < CH) L <<= 1;
    const int G = 32 / L, grp = lane / L, j = lane % L;
    uint32_t* wacc = sm + warp * (2 * S * rwp);
    uint32_t* wnew = wacc + S * rwp;

    const uint32_t* __restrict__ fin = d.front + (size_t)nx * d.C * S * rwp;
    const uint8_t* __restrict__ fflag_in = d.fflag + (size_t)nx * d.C;
    uint32_t* mplane = d.marked + (size_t)col * d.C * rwp;
    uint32_t* fout = d.front + (size_t)col * d.C * S * rwp;
    uint8_t* fflag_out = d.fflag + (size_t)col * d.C;
    const uint32_t* __restrict__ rp = d.g.row_ptr;
    const uint16_t* __restrict__ adj = d.g.col;
    const int np1 = n + 1;

    unsigned cnt = 0, err = 0;
    int wlo = kEmptyLo, whi = -1;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t cid = blockIdx.x * (blockDim.x >> 5) + warp; cid < d.C; cid += nwarps) {
        uint32_t* mrow = mplane + (size_t)cid * rwp;
        const uint32_t vm = lane < rw ? valid_mask(n, lane) : 0u;
        const uint32_t m = lane < rw ? mrow[lane] : 0u;
        if (__all_sync(FULL_MASK, m == vm)) continue;  // every robber position is marked

        Vec<VW> acc;
        acc.zero();
        if (direct) {
            if (grp == 0 && j < CH && fflag_in[cid]) acc.load_or(fin + (size_t)cid * S * rwp + j * VW);
        } else {
            const uint16_t* cc = d.configs + (size_t)cid * K;
            int lo[K], dg[K];
            int T = 1;
#pragma unroll
            for (int i = 0; i < K; ++i) {
                int v = cc[i];
                lo[i] = __ldg(&rp[v]);
                dg[i] = __ldg(&rp[v + 1]) - lo[i];
                T *= dg[i];
            }
            for (int t0 = 0; t0 < T; t0 += G) {
                const int t = t0 + grp;
                if (t < T && j < CH) {
                    int c[K];
                    int rem = t;
#pragma unroll
                    for (int i = K - 1; i >= 0; --i) {
                        int q = rem / dg[i];
                        c[i] = __ldg(&adj[lo[i] + rem - q * dg[i]]);
                        rem = q;
                    }
                    sort_small<K>(c);
                    const uint32_t s = config_rank<K>(c, d.binom, np1);
                    if (__ldg(&fflag_in[s])) acc.load_or(fin + (size_t)s * S * rwp + j * VW);
                }
            }
#pragma unroll
            for (int e = 0; e < VW; ++e)
                for (int off = L; off < 32; off <<= 1) acc.v[e] |= __shfl_xor_sync(FULL_MASK, acc.v[e], off);
        }
        if (grp == 0 && j < CH) {
#pragma unroll
            for (int e = 0; e < VW; ++e) wacc[j * VW + e] = acc.v[e];
        }
        __syncwarp();
        uint32_t mm = m, any = 0;
        if (lane < rw) {
            for (int s = 0; s < s_used; ++s) {
                const int v = base_in + s + 1;
                uint32_t nb = (v < kMaxRound) ? (wacc[s * rwp + lane] & ~mm & vm) : 0u;
                mm |= nb;
                wnew[s * rwp + lane] = nb;
                any |= nb;
                if (nb) { wlo = min(wlo, v); whi = max(whi, v); }
            }
        }
        __syncwarp();
        if (__any_sync(FULL_MASK, any != 0)) {
            if (lane < rw) {
                mrow[lane] = mm;
                cnt += __popc(mm ^ m);
            }
            uint32_t* frow = fout + (size_t)cid * S * rwp;
            for (int e = lane; e < S * rwp; e += 32) {
                const int so = e / rwp, w = e - so * rwp;
                const int s = out_base + so - base_in - 1;
                uint32_t val = (s >= 0 && s < s_used && w < rw) ? wnew[s * rwp + w] : 0u;
                frow[e] = append ? (frow[e] | val) : val;
            }
            if (lane < rw) {
                for (int s = 0; s < s_used; ++s) {
                    const int so = base_in + s + 1 - out_base;
                    if (wnew[s * rwp + lane] && (so < 0 || so >= S)) err |= kErrSlot;
                }
            }
            if (lane == 0) fflag_out[cid] = 1;
            uint8_t* trow = d.table + (size_t)cid * n * d.cols + col;
            for (int r = lane; r < n; r += 32) {
                const int w = r >> 5;
                const uint32_t bit = 1u << (r & 31);
                for (int s = 0; s < s_used; ++s) {
                    if (wnew[s * rwp + w] & bit) {
                        trow[(size_t)r * d.cols] = (uint8_t)(1 | ((base_in + s + 1) << 1));
                        break;
                    }
                }
            }
        }
        __syncwarp();
    }
    cnt = __reduce_add_sync(FULL_MASK, cnt);
    wlo = __reduce_min_sync(FULL_MASK, wlo);
    whi = __reduce_max_sync(FULL_MASK, whi);
    err = __reduce_or_sync(FULL_MASK, err);
    if (lane == 0) {
        if (cnt) atomicAdd(d.pass_new, (unsigned long long)cnt);
        if (whi >= 0) {
            atomicMin(&d.meta[col].lo, wlo);
            atomicMax(&d.meta[col].hi, whi);
        }
        if (err) atomicOr(d.err, err);
    }
}

// Last column (robber move cashed out over the exact-p-hop cloud) from column 0.
// One warp per configuration whose column-0 row changed; rows are row-local, so the subset
// test "every vertex of hop(r) is marked" is a handful of word ops against column 0's row.
template <bool P1>
__global__ void __launch_bounds__(256) k_and(V1Dev d, int col) {
    extern __shared__ uint32_t sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n = d.g.n, rw = d.g.rw, rwp = d.g.rwp, S = d.S, cols = d.cols;
    const ColMeta mi = d.meta[0];
    if (mi.hi < mi.lo) return;
    const int out_base = d.meta[col].base;
    const int per_warp = 2 * rwp + S * rwp + (n + 3) / 4;
    uint32_t* wm0 = sm + warp * per_warp;
    uint32_t* wmc = wm0 + rwp;
    uint32_t* wnew = wmc + rwp;
    uint8_t* wval = reinterpret_cast<uint8_t*>(wnew + S * rwp);

    const uint8_t* __restrict__ fflag0 = d.fflag;
    const uint32_t* __restrict__ m0plane = d.marked;
    uint32_t* mplane = d.marked + (size_t)col * d.C * rwp;
    uint32_t* fout = d.front + (size_t)col * d.C * S * rwp;
    uint8_t* fflag_out = d.fflag + (size_t)col * d.C;
    const uint32_t* __restrict__ rp = d.g.row_ptr;
    const uint16_t* __restrict__ adj = d.g.col;

    unsigned cnt = 0, err = 0;
    int wlo = kEmptyLo, whi = -1;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t cid = blockIdx.x * (blockDim.x >> 5) + warp; cid < d.C; cid += nwarps) {
        if (!fflag0[cid]) continue;
        uint32_t* mrow = mplane + (size_t)cid * rwp;
        const uint32_t vm = lane < rw ? valid_mask(n, lane) : 0u;
        const uint32_t mc = lane < rw ? mrow[lane] : 0u;
        if (__all_sync(FULL_MASK, mc == vm)) continue;
        if (lane < rwp) {
            wm0[lane] = lane < rw ? m0plane[(size_t)cid * rwp + lane] : 0u;
            wmc[lane] = mc;
        }
        for (int e = lane; e < S * rwp; e += 32) wnew[e] = 0u;
        const uint8_t* trow = d.table + (size_t)cid * n * cols;
        for (int r = lane; r < n; r += 32) wval[r] = trow[(size_t)r * cols] >> 1;
        __syncwarp();
        for (int r = lane; r < n; r += 32) {
            if ((wmc[r >> 5] >> (r & 31)) & 1u) continue;
            int mx = 0;
            bool all = true;
            if (P1) {
                for (uint32_t e = __ldg(&rp[r]); e < __ldg(&rp[r + 1]); ++e) {
                    const int v = __ldg(&adj[e]);
                    if (!((wm0[v >> 5] >> (v & 31)) & 1u)) { all = false; break; }
                    mx = max(mx, (int)wval[v]);
                }
            } else {
                const uint32_t* h = d.hop + (size_t)r * rwp;
                for (int w = 0; w < rw && all; ++w) all = (__ldg(&h[w]) & ~wm0[w]) == 0u;
                if (all) {
                    for (int w = 0; w < rw; ++w) {
                        uint32_t b = __ldg(&h[w]);
                        while (b) {
                            const int v = w * 32 + __ffs(b) - 1;
                            b &= b - 1;
                            mx = max(mx, (int)wval[v]);
                        }
                    }
                }
            }
            if (!all) continue;
            const int v = mx + 1;
            if (v >= kMaxRound) continue;
            const int so = v - out_base;
            if (so < 0 || so >= S) { err |= kErrSlot; continue; }
            atomicOr(&wnew[so * rwp + (r >> 5)], 1u << (r & 31));
            d.table[((size_t)cid * n + r) * cols + col] = (uint8_t)(1 | (v << 1));
            wlo = min(wlo, v);
            whi = max(whi, v);
        }
        __syncwarp();
        uint32_t nb = 0;
        if (lane < rw)
            for (int s = 0; s < S; ++s) nb |= wnew[s * rwp + lane];
        if (__any_sync(FULL_MASK, nb != 0)) {
            if (lane < rw) {
                mrow[lane] = mc | nb;
                cnt += __popc(nb);
            }
            uint32_t* frow = fout + (size_t)cid * S * rwp;
            for (int e = lane; e < S * rwp; e += 32) frow[e] = wnew[e];
            if (lane == 0) fflag_out[cid] = 1;
        }
        __syncwarp();
    }
    cnt = __reduce_add_sync(FULL_MASK, cnt);
    wlo = __reduce_min_sync(FULL_MASK, wlo);
    whi = __reduce_max_sync(FULL_MASK, whi);
    err = __reduce_or_sync(FULL_MASK, err);
    if (lane == 0) {
        if (cnt) atomicAdd(d.pass_new, (unsigned long long)cnt);
        if (whi >= 0) {
            atomicMin(&d.meta[col].lo, wlo);
            atomicMax(&d.meta[col].hi, whi);
        }
        if (err) atomicOr(d.err, err);
    }
}

// findFinalResult (k_cops_visibility.cpp:301-331): key = worst << 32 | cid, minimised, is the
// first config (lowest id) among those with the strictly smallest worst case.
__global__ void k_verdict(const uint8_t* __restrict__ table, const uint32_t* __restrict__ m0,
                          uint32_t C, int n, int rw, int rwp, int cols,
                          unsigned long long* best) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t cid = blockIdx.x * (blockDim.x >> 5) + warp; cid < C; cid += nwarps) {
        const uint32_t vm = lane < rw ? valid_mask(n, lane) : 0u;
        const uint32_t m = lane < rw ? m0[(size_t)cid * rwp + lane] : 0u;
        if (!__all_sync(FULL_MASK, m == vm)) continue;
        int wc = 0;
        for (int r = lane; r < n; r += 32) wc = max(wc, (int)(table[((size_t)cid * n + r) * cols] >> 1));
        wc = __reduce_max_sync(FULL_MASK, wc);
        if (lane == 0) atomicMin(best, ((unsigned long long)wc << 32) | cid);
    }
}

// Marked-state count of one column (resolved states for the statistics).
__global__ void k_popcount(const uint32_t* __restrict__ plane, size_t words, unsigned long long* out) {
    unsigned long long c = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < words;
         i += (size_t)gridDim.x * blockDim.x)
        c += __popc(plane[i]);
    c = __reduce_add_sync(FULL_MASK, (unsigned)c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// ---------------------------------------------------------------- host-side launchers ---

size_t cop_smem_bytes(int S, int rwp) { return (size_t)8 * 2 * S * rwp * sizeof(uint32_t); }
size_t and_smem_bytes(int S, int rwp, int n) {
    return (size_t)8 * (2 * rwp + S * rwp + (n + 3) / 4) * sizeof(uint32_t);
}

template <int K, int VW>
static void launch_cop_t(const V1Dev& d, int col, int nx, int direct, int grid, cudaStream_t st) {
    k_cop<K, VW><<<grid, 256, cop_smem_bytes(d.S, d.g.rwp), st>>>(d, col, nx, direct);
}

template <int K>
static void launch_cop_k(const V1Dev& d, int col, int nx, int direct, int grid, cudaStream_t st) {
    const int vw = d.g.rwp >= 4 ? 4 : d.g.rwp;
    if (vw == 4) launch_cop_t<K, 4>(d, col, nx, direct, grid, st);
    else if (vw == 2) launch_cop_t<K, 2>(d, col, nx, direct, grid, st);
    else launch_cop_t<K, 1>(d, col, nx, direct, grid, st);
}

void launch_cop(const V1Dev& d, int col, int nx, int direct, int grid, cudaStream_t st) {
    switch (d.k) {
        case 1: launch_cop_k<1>(d, col, nx, direct, grid, st); break;
        case 2: launch_cop_k<2>(d, col, nx, direct, grid, st); break;
        case 3: launch_cop_k<3>(d, col, nx, direct, grid, st); break;
        default: launch_cop_k<4>(d, col, nx, direct, grid, st); break;
    }
}

void launch_and(const V1Dev& d, int col, bool p1, int grid, cudaStream_t st) {
    const size_t sm = and_smem_bytes(d.S, d.g.rwp, d.g.n);
    if (p1) k_and<true><<<grid, 256, sm, st>>>(d, col);
    else k_and<false><<<grid, 256, sm, st>>>(d, col);
}

void launch_prep(const V1Dev& d, int col, int nx, int grid, cudaStream_t st) {
    k_prep<<<grid, 256, 0, st>>>(d, col, nx);
}

void launch_init(const V1Dev& d, int grid, cudaStream_t st) { k_init<<<grid, 256, 0, st>>>(d, d.k); }

void launch_verdict(const V1Dev& d, int col0_only_cols, unsigned long long* best, int grid,
                    cudaStream_t st) {
    k_verdict<<<grid, 256, 0, st>>>(d.table, d.marked, d.C, d.g.n, d.g.rw, d.g.rwp,
                                    col0_only_cols, best);
}

void launch_verdict_raw(const uint8_t* table, const uint32_t* m0, uint32_t C, int n, int rw,
                        int rwp, int cols, unsigned long long* best, int grid, cudaStream_t st) {
    k_verdict<<<grid, 256, 0, st>>>(table, m0, C, n, rw, rwp, cols, best);
}

void launch_popcount(const uint32_t* plane, size_t words, unsigned long long* out, int grid,
                     cudaStream_t st) {
    k_popcount<<<grid, 256, 0, st>>>(plane, words, out);
}

int max_cop_blocks_per_sm(int k, int rwp, int S) {
    int nb = 0;
    const size_t sm = cop_smem_bytes(S, rwp);
    const int vw = rwp >= 4 ? 4 : rwp;
    cudaError_t e = cudaSuccess;
#define CR_OCC(KK, VV) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_cop<KK, VV>, 256, sm)
    if (k == 1) { if (vw == 4) CR_OCC(1, 4); else if (vw == 2) CR_OCC(1, 2); else CR_OCC(1, 1); }
    else if (k == 2) { if (vw == 4) CR_OCC(2, 4); else if (vw == 2) CR_OCC(2, 2); else CR_OCC(2, 1); }
    else if (k == 3) { if (vw == 4) CR_OCC(3, 4); else if (vw == 2) CR_OCC(3, 2); else CR_OCC(3, 1); }
    else { if (vw == 4) CR_OCC(4, 4); else if (vw == 2) CR_OCC(4, 2); else CR_OCC(4, 1); }
#undef CR_OCC
    if (e != cudaSuccess || nb < 1) nb = 1;
    return nb;
}

}  // namespace crgpu
