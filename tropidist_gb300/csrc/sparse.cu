// Sparse (weight-truncated) Rank DP on the GPU: device hash tables of packed states.
//
// A state is packed like the reference's C tables (cdist/sparse_dp.c:3-4): key | value << 56, the
// key being the partial parities of the row slots (at most 56).  A table lives in two forms:
//   - an array of its n packed states (any order; a table is a set), and
//   - an open-addressing hash index of capacity 2^lg (linear probing, EMPTY = all ones), holding the
//     same packed states, used for lookups.
// One column step (cdist/sparse_dp.py:338-403, NumpyTables.step) is three kernels:
//   clear  the new index;
//   step   for every old state (key, v): the old state itself, if it passes the closing-row filter
//          ((key & sel_mask) == sel_bits, then those bits cleared), the cap and the lookahead bound,
//          is inserted with atomicMin; its candidate key ^ upd with value v + w (from v < cap) goes
//          through the same filters; a candidate is "changed" when no old state with its key has a
//          value <= its own (looked up in the OLD index), it is inserted when it improves an old
//          state or when it is new and below keep_below;
//   compact  the new index's occupied slots into the new array.
// Because the step's result is a set of per-key minima, it does not depend on the order in which
// threads insert: the tables equal the reference's entry for entry (as sets).
#include "tg_common.cuh"
#include "tg_capi.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace tg {

#define SP_EMPTY 0xFFFFFFFFFFFFFFFFull
#define SP_KEYMASK ((1ull << 56) - 1)
#define SP_QW 720720ll          // the lookahead weights are multiples of 1/QW (cdist/sparse_dp.py:48)
#define SP_MAXCLS 48

struct BoundParams {
    int on;                     // 0: no lookahead
    int ncls;
    int K;
    int pad;
    int64_t extra;
    uint64_t tmask;
    uint64_t mask[SP_MAXCLS];
    int64_t w[SP_MAXCLS];
};

// ceil((extra + sum_c w_c * |(key ^ tmask) & mask_c|) / QW)   (cdist/sparse_dp.py:208-217)
__device__ __forceinline__ int64_t sp_hbound(const BoundParams &b, uint64_t key) {
    const uint64_t u = key ^ b.tmask;
    int64_t tot = b.extra;
    for (int c = 0; c < b.ncls; c++) tot += b.w[c] * (int64_t)__popcll(u & b.mask[c]);
    return (tot + SP_QW - 1) / SP_QW;
}

__device__ __forceinline__ bool sp_keep(const BoundParams &b, uint64_t key, uint32_t v) {
    return !b.on || (int64_t)v + sp_hbound(b, key) <= (int64_t)b.K;
}

__device__ __forceinline__ uint32_t sp_slot(uint64_t key, int lg) {
    return (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - lg));
}

// insert (key, v) keeping the smaller value; returns 1 if the key was new, 0 if present, -1 if the
// index is full (the error flag is raised by the caller)
__device__ __forceinline__ int sp_insert_min(unsigned long long *H, int lg, uint64_t key, uint32_t v) {
    const unsigned long long packed = key | ((unsigned long long)v << 56);
    const uint32_t mask = (1u << lg) - 1u;
    uint32_t i = sp_slot(key, lg);
    for (uint32_t probe = 0; probe <= mask; probe++) {
        unsigned long long cur = H[i];
        if (cur == SP_EMPTY) {
            unsigned long long prev = atomicCAS(H + i, SP_EMPTY, packed);
            if (prev == SP_EMPTY) return 1;
            cur = prev;
        }
        if ((cur & SP_KEYMASK) == key) {
            atomicMin(H + i, packed);
            return 0;
        }
        i = (i + 1) & mask;
    }
    return -1;
}

// value of key in the index (255 = absent)
__device__ __forceinline__ uint32_t sp_lookup(const unsigned long long *H, int lg, uint64_t key) {
    if (!H) return 255;
    const uint32_t mask = (1u << lg) - 1u;
    uint32_t i = sp_slot(key, lg);
    for (uint32_t probe = 0; probe <= mask; probe++) {
        const unsigned long long cur = H[i];
        if (cur == SP_EMPTY) return 255;
        if ((cur & SP_KEYMASK) == key) return (uint32_t)(cur >> 56);
        i = (i + 1) & mask;
    }
    return 255;
}

__global__ void k_sp_fill(unsigned long long *H, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        H[i] = SP_EMPTY;
}

struct StepParams {
    uint64_t upd, sel_mask, sel_bits;
    int cap;                    // largest value kept
    int keep_below;             // new states with value >= keep_below go to `changed` only (-1: none)
    int w;                      // column weight (1 in the reference)
    int want_changed;
    int lg_old, lg_new;
};

// counters: [0] new keys inserted, [1] changed states, [2] error flags (1: index full, 2: changed overflow)
__global__ void k_sp_step(const __grid_constant__ StepParams P, const __grid_constant__ BoundParams B,
                          const unsigned long long *__restrict__ A, uint64_t n, const unsigned long long *Hold,
                          unsigned long long *Hnew, unsigned long long *changed, uint64_t changed_cap,
                          unsigned long long *counters) {
    const uint64_t clr = ~P.sel_mask & SP_KEYMASK;
    unsigned long long inserted = 0;      // new keys, added to counters[0] once at the end
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long x = A[i];
        const uint64_t key = x & SP_KEYMASK;
        const uint32_t v = (uint32_t)(x >> 56);
        // the old state
        if ((key & P.sel_mask) == P.sel_bits) {
            const uint64_t k2 = key & clr;
            if ((int)v <= P.cap && sp_keep(B, k2, v)) {
                const int r = sp_insert_min(Hnew, P.lg_new, k2, v);
                if (r > 0) inserted++;
                else if (r < 0) atomicOr(counters + 2, 1ull);
            }
        }
        // its candidate through the column
        if (P.upd && (int)v < P.cap) {
            const uint64_t t = key ^ P.upd;
            const uint32_t vc = v + (uint32_t)P.w;
            if ((t & P.sel_mask) == P.sel_bits) {
                const uint64_t t2 = t & clr;
                if ((int)vc <= P.cap && sp_keep(B, t2, vc)) {
                    const uint32_t vo = sp_lookup(Hold, P.lg_old, t);
                    const bool hit = vo != 255u;
                    if (vc < vo && P.want_changed) {
                        const unsigned long long slot = agg_inc(counters + 1);
                        if (slot < changed_cap) changed[slot] = t2 | ((unsigned long long)vc << 56);
                        else atomicOr(counters + 2, 2ull);
                    }
                    if (hit || P.keep_below < 0 || (int)vc < P.keep_below) {
                        const int r = sp_insert_min(Hnew, P.lg_new, t2, vc);
                        if (r > 0) inserted++;
                        else if (r < 0) atomicOr(counters + 2, 1ull);
                    }
                }
            }
        }
    }
    agg_add(counters + 0, inserted);
}

// the occupied slots of an index into an array; counters[3] = states written
__global__ void k_sp_compact(const unsigned long long *__restrict__ H, uint64_t cap, unsigned long long *out,
                             uint64_t out_cap, unsigned long long *counters) {
    // tiles of SPC_PER slots per thread: output positions are claimed once per block and tile
    constexpr int SPC_PER = 8;
    unsigned phase = 0;
    const uint64_t tile = (uint64_t)blockDim.x * SPC_PER;
    for (uint64_t t0 = blockIdx.x * tile; t0 < cap; t0 += (uint64_t)gridDim.x * tile) {
        unsigned long long x[SPC_PER];
        unsigned cnt = 0;
#pragma unroll
        for (int q = 0; q < SPC_PER; q++) {
            const uint64_t i = t0 + (uint64_t)q * blockDim.x + threadIdx.x;
            x[q] = i < cap ? H[i] : SP_EMPTY;
            cnt += x[q] != SP_EMPTY;
        }
        unsigned long long s, unused;
        block_claim2_n(phase, counters + 3, cnt, nullptr, 0u, s, unused);
#pragma unroll
        for (int q = 0; q < SPC_PER; q++) {
            if (x[q] == SP_EMPTY) continue;
            if (s < out_cap) out[s] = x[q];
            else atomicOr(counters + 2, 4ull);
            s++;
        }
    }
}

// index of an array of distinct packed states (values kept; entries with value >= below dropped
// from the copy written to `kept` when below >= 0)
__global__ void k_sp_build(const unsigned long long *__restrict__ A, uint64_t n, unsigned long long *H, int lg,
                           int below, unsigned long long *kept, unsigned long long *counters) {
    unsigned phase = 0;
    for (uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x; t0 < n; t0 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = t0 + threadIdx.x;
        const unsigned long long x = i < n ? A[i] : SP_EMPTY;
        const bool want = i < n && !(below >= 0 && (int)(x >> 56) >= below);
        if (kept) {
            const unsigned long long j = block_claim(phase, counters + 3, want);
            if (want) kept[j] = x;
        }
        if (!want) continue;
        const int r = sp_insert_min(H, lg, x & SP_KEYMASK, (uint32_t)(x >> 56));
        if (r < 0) atomicOr(counters + 2, 1ull);
    }
}

// join (cdist/sparse_dp.c:207-236): least f.value + b.value over changed forward states f and
// backward states b with key(b) = key(f) ^ tmask; result packed (total << 56 | forward key), the
// smallest total and, among equal totals, the smallest forward key
__global__ void k_sp_join(const unsigned long long *__restrict__ F, uint64_t nf, const unsigned long long *Hb, int lgb,
                          uint64_t tmask, unsigned long long *result) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nf; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long x = F[i];
        const uint64_t key = x & SP_KEYMASK;
        const uint32_t bv = sp_lookup(Hb, lgb, key ^ tmask);
        if (bv != 255u) {
            const unsigned long long tot = (x >> 56) + bv;
            atomicMin(result, (tot << 56) | key);
        }
    }
}

__global__ void k_sp_lookup(const unsigned long long *H, int lg, const unsigned long long *keys, uint64_t n,
                            uint8_t *vals) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        vals[i] = (uint8_t)sp_lookup(H, lg, keys[i] & SP_KEYMASK);
}

// value histogram of an array (hist[256], values 0..255)
__global__ void k_sp_hist(const unsigned long long *__restrict__ A, uint64_t n, unsigned long long *hist) {
    __shared__ unsigned int loc[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) loc[i] = 0;
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&loc[A[i] >> 56], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        if (loc[i]) atomicAdd(hist + i, (unsigned long long)loc[i]);
}

static unsigned sp_grid(uint64_t items) {
    uint64_t g = (items + 255) / 256;
    uint64_t cap = (uint64_t)sm_count() * 16;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

static int load_bound(BoundParams &B, int on, int K, int ncls, const uint64_t *masks, const int64_t *w, int64_t extra,
                      uint64_t tmask) {
    memset(&B, 0, sizeof(B));
    B.on = on;
    B.K = K;
    B.extra = extra;
    B.tmask = tmask;
    if (!on) return TG_OK;
    if (ncls < 0 || ncls > SP_MAXCLS) return set_error(TG_ERR_TOO_BIG, "more lookahead classes than the kernel holds");
    B.ncls = ncls;
    for (int c = 0; c < ncls; c++) { B.mask[c] = masks[c]; B.w[c] = w[c]; }
    return TG_OK;
}


// ------------------------------------------------------------------ walks: many steps per call
// Host-side loop over a run of column steps with the tables in caller-provided scratch (three
// table slots, a changed list), the kept tables copied into a caller-provided arena, and joins
// against backward indexes accumulated per step on the device: one call per run of steps instead
// of one per column, and no allocation.
#define SPW_FIELDS 16
#define SPW_KEEP_SMALL 1024             // keep flag 2: keep the table if it has at most this many states
enum { SW_UPD, SW_SELM, SW_SELB, SW_TMASK, SW_JTAB, SW_JTMASK, SW_EXTRA, SW_CAP, SW_KB, SW_W, SW_WANT, SW_TRUNC,
       SW_KEEP, SW_JLG, SW_NCLS, SW_USEH };

__host__ __device__ static int lg_for(uint64_t n) {  // index size for up to n states at load <= 1/2 (>= 64 slots)
    const uint64_t x = 2 * (n ? n : 1) - 1;
    int b = 0;
    while ((x >> b) != 0) b++;
    return b + 1 > 6 ? b + 1 : 6;
}

__global__ void k_sp_join_acc(const unsigned long long *__restrict__ F, uint64_t nf, const unsigned long long *Hb,
                              int lgb, uint64_t tmask, unsigned long long *result) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nf; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long x = F[i];
        const uint64_t key = x & SP_KEYMASK;
        const uint32_t bv = sp_lookup(Hb, lgb, key ^ tmask);
        if (bv != 255u) atomicMin(result, (((x >> 56) + bv) << 56) | key);
    }
}

// ---- small tables: one block runs many steps per launch (no host round trip per column)
#define SPW_SMALL_MAX 4096              // states per table in the one-block walk
#define SPW_SMALL_THREADS 1024

struct WalkSmall {
    const int64_t *spec;                // device copies of the walk's rows, lookahead classes
    const uint64_t *masks;
    const int64_t *weights;
    int stride, K, i0, nsteps;
    const unsigned long long *A0, *H0;  // the table before step i0
    uint64_t n0;
    int lg0, slot0;                     // slot0: scratch slot of that table (-1: outside the scratch)
    unsigned long long *arr[3], *idx[3], *changed;
    unsigned long long *arena;
    uint64_t arena_bytes, used0;
    int64_t *out;                       // device int64 [nsteps][6]
    unsigned long long *res;
    unsigned long long *state;          // out: [0] next step, [1] slot, [2] n, [3] lg, [4] arena used, [5] stop reason
};

// ---- tiny tables: the same steps with the working tables in shared memory
// The three scratch slots (states and index), the changed list and a copy of the join table live
// in shared memory, so a step touches global memory only for its outputs, kept tables and large
// join tables; the next step's rows are fetched while the current step runs.  It takes tables of at
// most SPW_TINY_N / 2 states with an index of at most 2^SPW_TINY_LG slots and stops (reason 1) when
// a step would need more; the table it ends with is written back to its global scratch slot.
#define SPW_TINY_N 1024
#define SPW_TINY_LG 12
#define SPW_TINY_THREADS 512
#define SPW_TINY_SMEM (8 * (3 * SPW_TINY_N + 3 * (1 << SPW_TINY_LG) + SPW_TINY_N + (1 << SPW_TINY_LG)))

__global__ void __launch_bounds__(SPW_TINY_THREADS) k_sp_walk_tiny(const __grid_constant__ WalkSmall P) {
    extern __shared__ unsigned long long sm_tiny[];
    auto sA = [&](int k) { return sm_tiny + k * SPW_TINY_N; };
    auto sH = [&](int k) { return sm_tiny + 3 * SPW_TINY_N + k * (1 << SPW_TINY_LG); };
    unsigned long long *sCH = sm_tiny + 3 * SPW_TINY_N + 3 * (1 << SPW_TINY_LG);
    unsigned long long *sJ = sCH + SPW_TINY_N;
    __shared__ unsigned long long c_ch, c_out, c_tr, c_flag;
    __shared__ BoundParams B[2];
    __shared__ int64_t F[2][SPW_FIELDS];
    __shared__ const unsigned long long *j_cached;
    const unsigned tid = threadIdx.x, NT = blockDim.x;
    int cur = P.slot0;
    int sc = cur >= 0 ? cur : 2;          // shared slot of the current table (an outside table goes to 2)
    uint64_t n = P.n0;
    int lg = P.lg0;
    uint64_t used = P.used0;
    int i = P.i0, reason = 0;
    // the table before step i0, and the rows of step i0
    for (uint64_t k = tid; k < n; k += NT) sA(sc)[k] = P.A0[k];
    for (uint64_t k = tid; k < (1ull << lg); k += NT) sH(sc)[k] = P.H0[k];
    auto load_rows = [&](int step, int buf) {
        const int64_t *f = P.spec + (size_t)SPW_FIELDS * step;
        if (tid < SPW_FIELDS) F[buf][tid] = f[tid];
        const int nc = (int)f[SW_NCLS];
        for (int c = tid; c < nc && c < SP_MAXCLS; c += NT) {
            B[buf].mask[c] = P.masks[(size_t)P.stride * step + c];
            B[buf].w[c] = P.weights[(size_t)P.stride * step + c];
        }
        if (tid == 0) {
            B[buf].on = (int)f[SW_USEH];
            B[buf].ncls = nc;
            B[buf].K = P.K;
            B[buf].extra = f[SW_EXTRA];
            B[buf].tmask = (uint64_t)f[SW_TMASK];
        }
    };
    if (i < P.nsteps) load_rows(i, i & 1);
    if (tid == 0) { c_ch = c_out = c_tr = c_flag = 0; j_cached = nullptr; }
    __syncthreads();
    for (; i < P.nsteps; i++) {
        const int b = i & 1;
        const int64_t *f = F[b];
        if (2 * n > SPW_TINY_N) { reason = 1; break; }
        int os = 0;
        while (os == cur) os++;
        const int lgn = lg_for(2 * n);
        const uint64_t capn = 1ull << lgn;
        unsigned long long *H = sH(os), *A = sA(os);
        for (uint64_t k = tid; k < capn; k += NT) H[k] = SP_EMPTY;
        // the next step's rows: loads issued now, stored at the end of the step
        int64_t pf = 0;
        uint64_t pm = 0;
        int64_t pw = 0;
        const bool more = i + 1 < P.nsteps;
        if (more) {
            const int64_t *fn = P.spec + (size_t)SPW_FIELDS * (i + 1);
            if (tid < SPW_FIELDS) pf = fn[tid];
            if (tid >= 32 && tid < 32 + (unsigned)SP_MAXCLS && (int)(tid - 32) < P.stride) {
                pm = P.masks[(size_t)P.stride * (i + 1) + (tid - 32)];
                pw = P.weights[(size_t)P.stride * (i + 1) + (tid - 32)];
            }
        }
        // a join table small enough is copied once and then probed in shared memory
        const unsigned long long *jG = reinterpret_cast<const unsigned long long *>((uintptr_t)f[SW_JTAB]);
        const int jlg = (int)f[SW_JLG];
        const bool jS = jG && jlg <= SPW_TINY_LG;
        if (jS && j_cached != jG)
            for (uint64_t k = tid; k < (1ull << jlg); k += NT) sJ[k] = jG[k];
        __syncthreads();
        if (tid == 0 && jS) j_cached = jG;
        const unsigned long long *curA = sA(sc), *curH = sH(sc);
        const uint64_t upd = (uint64_t)f[SW_UPD] & SP_KEYMASK, selm = (uint64_t)f[SW_SELM], selb = (uint64_t)f[SW_SELB];
        const uint64_t clr = ~selm & SP_KEYMASK;
        const int cap = (int)f[SW_CAP], kb = (int)f[SW_KB], w = (int)f[SW_W];
        const bool want = f[SW_WANT] != 0;
        for (uint64_t k = tid; k < n; k += NT) {
            const unsigned long long x = curA[k];
            const uint64_t key = x & SP_KEYMASK;
            const uint32_t v = (uint32_t)(x >> 56);
            if ((key & selm) == selb) {
                const uint64_t k2 = key & clr;
                if ((int)v <= cap && sp_keep(B[b], k2, v)) {
                    if (sp_insert_min(H, lgn, k2, v) < 0) atomicOr(&c_flag, 1ull);
                }
            }
            if (upd && (int)v < cap) {
                const uint64_t t = key ^ upd;
                const uint32_t vc = v + (uint32_t)w;
                if ((t & selm) == selb) {
                    const uint64_t t2 = t & clr;
                    if ((int)vc <= cap && sp_keep(B[b], t2, vc)) {
                        const uint32_t vo = sp_lookup(curH, lg, t);
                        const bool hit = vo != 255u;
                        if (vc < vo && want) {
                            const unsigned long long q = atomicAdd(&c_ch, 1ull);
                            if (q < SPW_TINY_N) sCH[q] = t2 | ((unsigned long long)vc << 56);
                            else atomicOr(&c_flag, 1ull);
                        }
                        if (hit || kb < 0 || (int)vc < kb) {
                            if (sp_insert_min(H, lgn, t2, vc) < 0) atomicOr(&c_flag, 1ull);
                        }
                    }
                }
            }
        }
        __syncthreads();
        for (uint64_t k = tid; k < capn; k += NT) {
            const unsigned long long x = H[k];
            if (x != SP_EMPTY) {
                const unsigned long long q = atomicAdd(&c_out, 1ull);
                if (q < SPW_TINY_N) A[q] = x;
                else atomicOr(&c_flag, 1ull);
            }
        }
        __syncthreads();
        if (c_flag) { reason = 4; break; }
        uint64_t nn = c_out;
        const uint64_t nch = want ? c_ch : 0;
        const uint64_t jt = (uint64_t)f[SW_JTMASK] & SP_KEYMASK;
        const unsigned long long *jH = jS ? sJ : jG;
        unsigned long long best = ~0ull;
        if (jH)
            for (uint64_t k = tid; k < nch; k += NT) {
                const unsigned long long x = sCH[k];
                const uint32_t bv = sp_lookup(jH, jlg, (x & SP_KEYMASK) ^ jt);
                if (bv != 255u) best = min(best, (((x >> 56) + bv) << 56) | (x & SP_KEYMASK));
            }
        int64_t *o = P.out + 6 * (size_t)i;
        if (tid == 0) o[5] = (int64_t)nn;
        int nlg = lgn, ns = os;
        if (f[SW_TRUNC] >= 0) {
            if (jH)
                for (uint64_t k = tid; k < nn; k += NT) {
                    const unsigned long long x = A[k];
                    const uint32_t bv = sp_lookup(jH, jlg, (x & SP_KEYMASK) ^ jt);
                    if (bv != 255u) best = min(best, (((x >> 56) + bv) << 56) | (x & SP_KEYMASK));
                }
            int ts = 0;
            while (ts == os) ts++;
            const int lgt = lg_for(nn);
            unsigned long long *T = sH(ts), *TA = sA(ts);
            for (uint64_t k = tid; k < (1ull << lgt); k += NT) T[k] = SP_EMPTY;
            __syncthreads();
            const int below = (int)f[SW_TRUNC];
            for (uint64_t k = tid; k < nn; k += NT) {
                const unsigned long long x = A[k];
                if ((int)(x >> 56) >= below) continue;
                if (sp_insert_min(T, lgt, x & SP_KEYMASK, (uint32_t)(x >> 56)) < 0) atomicOr(&c_flag, 1ull);
                TA[atomicAdd(&c_tr, 1ull)] = x;
            }
            __syncthreads();
            nn = c_tr;
            nlg = lgt;
            ns = ts;
        }
        if (jH && best != ~0ull) atomicMin(P.res + i, best);
        int64_t a_off = -1, h_off = -1;
        if (f[SW_KEEP] == 1 || (f[SW_KEEP] == 2 && nn <= SPW_KEEP_SMALL)) {
            const int lgk = lg_for(nn);
            const uint64_t ab = (8 * nn + 255) / 256 * 256, ib = 8ull << lgk;
            if (used + ab + ib > P.arena_bytes) { reason = 2; break; }
            unsigned long long *kA = P.arena + used / 8, *kH = P.arena + (used + ab) / 8;
            const unsigned long long *nA = sA(ns);
            for (uint64_t k = tid; k < nn; k += NT) kA[k] = nA[k];
            for (uint64_t k = tid; k < (1ull << lgk); k += NT) kH[k] = SP_EMPTY;
            __syncthreads();
            for (uint64_t k = tid; k < nn; k += NT)
                if (sp_insert_min(kH, lgk, nA[k] & SP_KEYMASK, (uint32_t)(nA[k] >> 56)) < 0) atomicOr(&c_flag, 1ull);
            a_off = (int64_t)used;
            h_off = (int64_t)(used + ab);
            used += ab + ib;
            if (tid == 0) o[4] = lgk;
        } else if (tid == 0) {
            o[4] = nlg;
        }
        if (tid == 0) {
            o[0] = (int64_t)nn;
            o[1] = (int64_t)nch;
            o[2] = a_off;
            o[3] = h_off;
        }
        n = nn;
        lg = nlg;
        cur = ns;
        sc = ns;
        // the next step's rows (fetched above) into the other buffer
        if (more) {
            const int nb = b ^ 1;
            if (tid < SPW_FIELDS) F[nb][tid] = pf;
            if (tid >= 32 && tid < 32 + (unsigned)SP_MAXCLS && (int)(tid - 32) < P.stride) {
                B[nb].mask[tid - 32] = pm;
                B[nb].w[tid - 32] = pw;
            }
        }
        __syncthreads();
        if (tid == 0) {
            if (more) {
                B[b ^ 1].on = (int)F[b ^ 1][SW_USEH];
                B[b ^ 1].ncls = (int)F[b ^ 1][SW_NCLS];
                B[b ^ 1].K = P.K;
                B[b ^ 1].extra = F[b ^ 1][SW_EXTRA];
                B[b ^ 1].tmask = (uint64_t)F[b ^ 1][SW_TMASK];
            }
            c_ch = c_out = c_tr = 0;
        }
        __syncthreads();
    }
    // the current table back to its global scratch slot (the steps' results are all there)
    if (i > P.i0 && cur >= 0) {
        for (uint64_t k = tid; k < n; k += NT) P.arr[cur][k] = sA(sc)[k];
        for (uint64_t k = tid; k < (1ull << lg); k += NT) P.idx[cur][k] = sH(sc)[k];
    }
    if (tid == 0) {
        P.state[0] = (unsigned long long)i;
        P.state[1] = (unsigned long long)(long long)cur;
        P.state[2] = n;
        P.state[3] = (unsigned long long)lg;
        P.state[4] = used;
        P.state[5] = (unsigned long long)reason;
    }
}

// stop reasons: 1 a table beyond SPW_SMALL_MAX (continue with the per-step path), 2 arena full,
// 4 index full, 5 the tables fit the shared-memory walk again
__global__ void __launch_bounds__(SPW_SMALL_THREADS) k_sp_walk_small(const __grid_constant__ WalkSmall P) {
    __shared__ unsigned long long c_ch, c_out, c_flag;
    __shared__ BoundParams B;
    const unsigned long long *curA = P.A0, *curH = P.H0;
    uint64_t n = P.n0;
    int lg = P.lg0, cur = P.slot0;
    uint64_t used = P.used0;
    int i = P.i0, reason = 0;
    const unsigned tid = threadIdx.x, NT = blockDim.x;
    for (; i < P.nsteps; i++) {
        const int64_t *f = P.spec + (size_t)SPW_FIELDS * i;
        if (2 * n > SPW_SMALL_MAX) { reason = 1; break; }
        if (i > P.i0 && 4 * 2 * n <= SPW_TINY_N && lg <= SPW_TINY_LG) { reason = 5; break; }
        int os = 0;
        while (os == cur) os++;
        const int lgn = lg_for(2 * n);
        const uint64_t capn = 1ull << lgn;
        if (tid == 0) {
            c_ch = c_out = c_flag = 0;
            B.on = (int)f[SW_USEH];
            B.ncls = (int)f[SW_NCLS];
            B.K = P.K;
            B.extra = f[SW_EXTRA];
            B.tmask = (uint64_t)f[SW_TMASK];
        }
        for (int c = tid; c < (int)f[SW_NCLS] && c < SP_MAXCLS; c += NT) {
            B.mask[c] = P.masks[(size_t)P.stride * i + c];
            B.w[c] = P.weights[(size_t)P.stride * i + c];
        }
        unsigned long long *H = P.idx[os];
        for (uint64_t k = tid; k < capn; k += NT) H[k] = SP_EMPTY;
        __syncthreads();
        const uint64_t upd = (uint64_t)f[SW_UPD] & SP_KEYMASK, selm = (uint64_t)f[SW_SELM], selb = (uint64_t)f[SW_SELB];
        const uint64_t clr = ~selm & SP_KEYMASK;
        const int cap = (int)f[SW_CAP], kb = (int)f[SW_KB], w = (int)f[SW_W];
        const bool want = f[SW_WANT] != 0;
        for (uint64_t k = tid; k < n; k += NT) {
            const unsigned long long x = curA[k];
            const uint64_t key = x & SP_KEYMASK;
            const uint32_t v = (uint32_t)(x >> 56);
            if ((key & selm) == selb) {
                const uint64_t k2 = key & clr;
                if ((int)v <= cap && sp_keep(B, k2, v)) {
                    const int r = sp_insert_min(H, lgn, k2, v);
                    if (r < 0) atomicOr(&c_flag, 1ull);
                }
            }
            if (upd && (int)v < cap) {
                const uint64_t t = key ^ upd;
                const uint32_t vc = v + (uint32_t)w;
                if ((t & selm) == selb) {
                    const uint64_t t2 = t & clr;
                    if ((int)vc <= cap && sp_keep(B, t2, vc)) {
                        const uint32_t vo = sp_lookup(curH, lg, t);
                        const bool hit = vo != 255u;
                        if (vc < vo && want) P.changed[atomicAdd(&c_ch, 1ull)] = t2 | ((unsigned long long)vc << 56);
                        if (hit || kb < 0 || (int)vc < kb) {
                            const int r = sp_insert_min(H, lgn, t2, vc);
                            if (r < 0) atomicOr(&c_flag, 1ull);
                        }
                    }
                }
            }
        }
        __syncthreads();
        unsigned long long *A = P.arr[os];
        for (uint64_t k = tid; k < capn; k += NT) {
            const unsigned long long x = H[k];
            if (x != SP_EMPTY) A[atomicAdd(&c_out, 1ull)] = x;
        }
        __syncthreads();
        if (c_flag) { reason = 4; break; }
        uint64_t nn = c_out;
        const uint64_t nch = want ? c_ch : 0;
        __syncthreads();                // every thread has read the counters before they are reused
        const unsigned long long *jH = reinterpret_cast<const unsigned long long *>((uintptr_t)f[SW_JTAB]);
        const uint64_t jt = (uint64_t)f[SW_JTMASK] & SP_KEYMASK;
        const int jlg = (int)f[SW_JLG];
        unsigned long long best = ~0ull;
        if (jH)
            for (uint64_t k = tid; k < nch; k += NT) {
                const unsigned long long x = P.changed[k];
                const uint32_t bv = sp_lookup(jH, jlg, (x & SP_KEYMASK) ^ jt);
                if (bv != 255u) best = min(best, (((x >> 56) + bv) << 56) | (x & SP_KEYMASK));
            }
        int64_t *o = P.out + 6 * (size_t)i;
        if (tid == 0) o[5] = (int64_t)nn;
        const unsigned long long *nA = A, *nH = H;
        int nlg = lgn, ns = os;
        if (f[SW_TRUNC] >= 0) {
            if (jH)
                for (uint64_t k = tid; k < nn; k += NT) {
                    const unsigned long long x = A[k];
                    const uint32_t bv = sp_lookup(jH, jlg, (x & SP_KEYMASK) ^ jt);
                    if (bv != 255u) best = min(best, (((x >> 56) + bv) << 56) | (x & SP_KEYMASK));
                }
            int ts = 0;
            while (ts == os) ts++;
            const int lgt = lg_for(nn);
            unsigned long long *T = P.idx[ts], *TA = P.arr[ts];
            for (uint64_t k = tid; k < (1ull << lgt); k += NT) T[k] = SP_EMPTY;
            if (tid == 0) c_out = 0;
            __syncthreads();
            const int below = (int)f[SW_TRUNC];
            for (uint64_t k = tid; k < nn; k += NT) {
                const unsigned long long x = A[k];
                if ((int)(x >> 56) >= below) continue;
                if (sp_insert_min(T, lgt, x & SP_KEYMASK, (uint32_t)(x >> 56)) < 0) atomicOr(&c_flag, 1ull);
                TA[atomicAdd(&c_out, 1ull)] = x;
            }
            __syncthreads();
            nn = c_out;
            nA = TA;
            nH = T;
            nlg = lgt;
            ns = ts;
        }
        if (jH && best != ~0ull) atomicMin(P.res + i, best);
        int64_t a_off = -1, h_off = -1;
        if (f[SW_KEEP] == 1 || (f[SW_KEEP] == 2 && nn <= SPW_KEEP_SMALL)) {
            const int lgk = lg_for(nn);
            const uint64_t ab = (8 * nn + 255) / 256 * 256, ib = 8ull << lgk;
            if (used + ab + ib > P.arena_bytes) { reason = 2; break; }
            unsigned long long *kA = P.arena + used / 8, *kH = P.arena + (used + ab) / 8;
            for (uint64_t k = tid; k < nn; k += NT) kA[k] = nA[k];
            for (uint64_t k = tid; k < (1ull << lgk); k += NT) kH[k] = SP_EMPTY;
            __syncthreads();
            for (uint64_t k = tid; k < nn; k += NT)
                if (sp_insert_min(kH, lgk, kA[k] & SP_KEYMASK, (uint32_t)(kA[k] >> 56)) < 0) atomicOr(&c_flag, 1ull);
            a_off = (int64_t)used;
            h_off = (int64_t)(used + ab);
            used += ab + ib;
            if (tid == 0) o[4] = lgk;   // the working index stays the table's index for the next step
        } else if (tid == 0) {
            o[4] = nlg;
        }
        if (tid == 0) {
            o[0] = (int64_t)nn;
            o[1] = (int64_t)nch;
            o[2] = a_off;
            o[3] = h_off;
        }
        curA = nA;
        curH = nH;
        n = nn;
        lg = nlg;
        cur = ns;
        __syncthreads();
    }
    if (tid == 0) {
        P.state[0] = (unsigned long long)i;
        P.state[1] = (unsigned long long)(long long)cur;
        P.state[2] = n;
        P.state[3] = (unsigned long long)lg;
        P.state[4] = used;
        P.state[5] = (unsigned long long)reason;
    }
}

struct WalkScratch {
    uint64_t cap_n;
    int lgc;
    unsigned long long *arr[3], *idx[3], *changed;
};

static uint64_t walk_scratch_bytes(uint64_t cap_n, int &lgc) {
    lgc = lg_for(cap_n);
    return 8 * (4 * cap_n + 3 * (1ull << lgc));
}

static bool walk_layout(void *scratch, uint64_t cap_n, WalkScratch &W) {
    W.cap_n = cap_n;
    walk_scratch_bytes(cap_n, W.lgc);
    unsigned long long *p = static_cast<unsigned long long *>(scratch);
    for (int k = 0; k < 3; k++) { W.arr[k] = p; p += cap_n; }
    W.changed = p;
    p += cap_n;
    for (int k = 0; k < 3; k++) { W.idx[k] = p; p += 1ull << W.lgc; }
    return true;
}

}  // namespace tg

using namespace tg;

extern "C" {

// Fill an index with EMPTY.
int tg_sp_clear(void *H, uint64_t cap, void *stream) {
    if (!H || cap == 0) return set_error(TG_ERR_ARG, "null index");
    k_sp_fill<<<sp_grid(cap), 256, 0, (cudaStream_t)stream>>>((unsigned long long *)H, cap);
    return cuda_check(cudaGetLastError(), "sparse clear");
}

// One column step (see the file comment).  A: old array (n states), Hold: old index (2^lg_old
// slots, may be null when n == 0 or upd == 0), Hnew: new index (2^lg_new slots, cleared by the
// call), Anew: new array (room for anew_cap), changed: changed states (room for changed_cap);
// counters (device, 4 x uint64): zeroed by the call; [0] new keys, [1] changed, [2] error flags,
// [3] states in Anew.  bound: ncls classes (masks, weights in 1/720720 units), extra, tmask, K.
int tg_sp_step(const void *A, uint64_t n, const void *Hold, int lg_old, void *Hnew, int lg_new, void *Anew,
               uint64_t anew_cap, void *changed, uint64_t changed_cap, uint64_t upd, uint64_t sel_mask,
               uint64_t sel_bits, int cap, int keep_below, int w, int want_changed, int use_h, int K, int ncls,
               const uint64_t *masks, const int64_t *weights, int64_t extra, uint64_t tmask, void *counters,
               void *stream) {
    if (lg_new < 1 || lg_new > 40 || (n && !A) || !Hnew || !Anew || !counters) return set_error(TG_ERR_ARG, "bad sparse step");
    if (cap > 254 || w < 1 || w > 254) return set_error(TG_ERR_ARG, "values beyond 8 bits");
    StepParams P;
    P.upd = upd & SP_KEYMASK;
    P.sel_mask = sel_mask;
    P.sel_bits = sel_bits;
    P.cap = cap;
    P.keep_below = keep_below;
    P.w = w;
    P.want_changed = want_changed && changed;
    P.lg_old = lg_old;
    P.lg_new = lg_new;
    BoundParams B;
    int e = load_bound(B, use_h, K, ncls, masks, weights, extra, tmask);
    if (e) return e;
    cudaStream_t st = (cudaStream_t)stream;
    e = cuda_check(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned long long), st), "counters");
    if (e) return e;
    const uint64_t capn = 1ull << lg_new;
    k_sp_fill<<<sp_grid(capn), 256, 0, st>>>((unsigned long long *)Hnew, capn);
    if (n) k_sp_step<<<sp_grid(n), 256, 0, st>>>(P, B, (const unsigned long long *)A, n, (const unsigned long long *)Hold,
                                                (unsigned long long *)Hnew, (unsigned long long *)changed, changed_cap,
                                                (unsigned long long *)counters);
    k_sp_compact<<<sp_grid((capn + 7) / 8), 256, 0, st>>>((const unsigned long long *)Hnew, capn, (unsigned long long *)Anew,
                                                anew_cap, (unsigned long long *)counters);
    return cuda_check(cudaGetLastError(), "sparse step");
}

// Bytes of scratch for a walk whose tables hold up to cap_n states (three table slots with their
// indexes and a changed list).
int64_t tg_sp_walk_scratch_bytes(uint64_t cap_n) {
    int lgc;
    return (int64_t)walk_scratch_bytes(cap_n, lgc);
}

// A run of nsteps column steps from the table (A0, n0, H0, lg0) (device; left unchanged).
// spec: host int64[nsteps][16]: upd, sel_mask, sel_bits, lookahead tmask, join index (device
// pointer, 0: no join), join tmask, lookahead extra, cap, keep_below (-1: none), w, want_changed,
// trunc_below (-1: none; else the table after the step keeps values < trunc_below and the table
// before is joined in full), keep, join lg, ncls, use_h.  masks / weights: host [nsteps][stride]
// lookahead classes.  scratch: tg_sp_walk_scratch_bytes(cap_n) bytes.  Kept tables are copied into
// the arena (array, then index, 256-byte aligned).  out: host int64[nsteps][6]: states after the
// step, changed states, arena byte offsets of the kept array and index (-1: not kept), index lg,
// states before truncation.  join_results: device uint64[nsteps], each the packed minimum
// (total << 56 | forward key) of the step's joins (all ones: no pair).  Returns nsteps, or the
// step at which the scratch (need[0]: states per table) or the arena (need[1]: bytes) ran out
// (nothing of the run is usable then: run it again with more room); negative status on errors.
int tg_sp_walk(int nsteps, const int64_t *spec, const uint64_t *masks, const int64_t *weights, int stride, int K,
               const void *A0, uint64_t n0, const void *H0, int lg0, void *scratch, uint64_t cap_n, void *arena,
               uint64_t arena_bytes, int64_t *out, void *join_results, int64_t *need, void *counters, void *stream) {
    if (nsteps < 0 || (nsteps && !spec) || !out || !scratch || !counters || (n0 && (!A0 || !H0)) ||
        (nsteps && !join_results) || !need || cap_n < 2)
        return set_error(TG_ERR_ARG, "bad walk");
    cudaStream_t st = (cudaStream_t)stream;
    WalkScratch W;
    walk_layout(scratch, cap_n, W);
    unsigned long long *cnt = static_cast<unsigned long long *>(counters);
    unsigned long long *res = static_cast<unsigned long long *>(join_results);
    static thread_local unsigned long long *hb = nullptr;        // pinned readback of the counters
    if (!hb && cudaMallocHost(&hb, 64) != cudaSuccess) {
        cudaGetLastError();
        hb = nullptr;
        return set_error(TG_ERR_NOMEM, "pinned walk buffer");
    }
    int e = TG_OK;
    if (nsteps) e = cuda_check(cudaMemsetAsync(res, 0xFF, 8 * (size_t)nsteps, st), "join init");
    if (e) return e;
    auto read_counters = [&]() -> int {
        int r = cuda_check(cudaMemcpyAsync(hb, cnt, 32, cudaMemcpyDeviceToHost, st), "walk counters");
        if (!r) r = cuda_check(cudaStreamSynchronize(st), "walk sync");
        if (!r && hb[2]) r = set_error(TG_ERR_STATE, "walk table overflow");
        return r;
    };
    const unsigned long long *curA = static_cast<const unsigned long long *>(A0);
    const unsigned long long *curH = static_cast<const unsigned long long *>(H0);
    uint64_t n = n0;
    int lg = lg0, cur = -1;
    uint64_t used = 0;
    need[0] = need[1] = 0;
    // device copies of the rows for the one-block walk of small tables
    static thread_local uint8_t *dbuf = nullptr;
    static thread_local size_t dbuf_bytes = 0;
    const size_t b_spec = 8 * (size_t)SPW_FIELDS * nsteps, b_cls = 8 * (size_t)stride * nsteps;
    const size_t b_out = 8 * 6 * (size_t)nsteps, b_all = b_spec + 2 * b_cls + b_out + 64;
    const bool small_ok = cap_n >= SPW_SMALL_MAX && nsteps > 0;
    if (small_ok) {
        if (dbuf_bytes < b_all) {
            if (dbuf) cudaFree(dbuf);
            dbuf = nullptr;
            dbuf_bytes = 0;
            if (cudaMalloc(&dbuf, b_all) != cudaSuccess) {
                cudaGetLastError();
                return set_error(TG_ERR_NOMEM, "walk rows");
            }
            dbuf_bytes = b_all;
        }
        e = cuda_check(cudaMemcpyAsync(dbuf, spec, b_spec, cudaMemcpyHostToDevice, st), "walk rows");
        if (!e && b_cls) e = cuda_check(cudaMemcpyAsync(dbuf + b_spec, masks, b_cls, cudaMemcpyHostToDevice, st), "walk rows");
        if (!e && b_cls) e = cuda_check(cudaMemcpyAsync(dbuf + b_spec + b_cls, weights, b_cls, cudaMemcpyHostToDevice, st), "walk rows");
        if (e) return e;
    }
    static bool tiny_attr = false;
    if (small_ok && !tiny_attr) {
        e = cuda_check(cudaFuncSetAttribute(k_sp_walk_tiny, cudaFuncAttributeMaxDynamicSharedMemorySize, SPW_TINY_SMEM),
                       "tiny walk shared memory");
        if (e) return e;
        tiny_attr = true;
    }
    for (int i = 0; i < nsteps; i++) {
        // one-block walks while the tables are small: shared-memory tables first, then global ones;
        // each stops when its tables outgrow it (the small walk also when they become tiny again)
        while (small_ok && i < nsteps && 2 * n <= SPW_SMALL_MAX) {
            const bool tiny = 2 * n <= SPW_TINY_N && lg <= SPW_TINY_LG;
            WalkSmall S;
            S.spec = reinterpret_cast<const int64_t *>(dbuf);
            S.masks = reinterpret_cast<const uint64_t *>(dbuf + b_spec);
            S.weights = reinterpret_cast<const int64_t *>(dbuf + b_spec + b_cls);
            S.stride = stride;
            S.K = K;
            S.i0 = i;
            S.nsteps = nsteps;
            S.A0 = curA;
            S.H0 = curH;
            S.n0 = n;
            S.lg0 = lg;
            S.slot0 = cur;
            for (int k = 0; k < 3; k++) { S.arr[k] = W.arr[k]; S.idx[k] = W.idx[k]; }
            S.changed = W.changed;
            S.arena = static_cast<unsigned long long *>(arena);
            S.arena_bytes = arena ? arena_bytes : 0;
            S.used0 = used;
            S.out = reinterpret_cast<int64_t *>(dbuf + b_spec + 2 * b_cls);
            S.res = res;
            unsigned long long *dstate = reinterpret_cast<unsigned long long *>(dbuf + b_spec + 2 * b_cls + b_out);
            S.state = dstate;
            if (tiny) k_sp_walk_tiny<<<1, SPW_TINY_THREADS, SPW_TINY_SMEM, st>>>(S);
            else k_sp_walk_small<<<1, SPW_SMALL_THREADS, 0, st>>>(S);
            e = cuda_check(cudaGetLastError(), "small walk");
            if (!e) e = cuda_check(cudaMemcpyAsync(hb, dstate, 48, cudaMemcpyDeviceToHost, st), "small walk state");
            if (!e) e = cuda_check(cudaMemcpyAsync(out + 6 * (size_t)i, S.out + 6 * (size_t)i, 48 * (size_t)(nsteps - i),
                                                   cudaMemcpyDeviceToHost, st), "small walk rows");
            if (!e) e = cuda_check(cudaStreamSynchronize(st), "small walk sync");
            if (e) return e;
            const int i1 = (int)hb[0];
            const int reason = (int)hb[5];
            if (i1 > i) {
                cur = (int)(long long)hb[1];
                n = hb[2];
                lg = (int)hb[3];
                used = hb[4];
                curA = W.arr[cur];
                curH = W.idx[cur];
            }
            if (reason == 2) { need[1] = (int64_t)(2 * arena_bytes + (1 << 20)); return i1; }
            if (reason == 4) return set_error(TG_ERR_STATE, "walk table overflow");
            const bool progressed = i1 > i;
            i = i1;
            if (!progressed && !tiny) break;    // the next step needs the per-step path
        }
        if (i >= nsteps) break;
        const int64_t *f = spec + (size_t)SPW_FIELDS * i;
        int64_t *o = out + 6 * (size_t)i;
        if (2 * n > cap_n) { need[0] = (int64_t)(2 * n); return i; }
        if (f[SW_CAP] > 254 || f[SW_W] < 1 || f[SW_W] > 254) return set_error(TG_ERR_ARG, "values beyond 8 bits");
        int os = 0;
        while (os == cur) os++;
        const int lgn = lg_for(2 * n);
        StepParams P;
        P.upd = (uint64_t)f[SW_UPD] & SP_KEYMASK;
        P.sel_mask = (uint64_t)f[SW_SELM];
        P.sel_bits = (uint64_t)f[SW_SELB];
        P.cap = (int)f[SW_CAP];
        P.keep_below = (int)f[SW_KB];
        P.w = (int)f[SW_W];
        P.want_changed = f[SW_WANT] != 0;
        P.lg_old = lg;
        P.lg_new = lgn;
        BoundParams B;
        e = load_bound(B, (int)f[SW_USEH], K, (int)f[SW_NCLS], masks + (size_t)stride * i, weights + (size_t)stride * i,
                       f[SW_EXTRA], (uint64_t)f[SW_TMASK]);
        if (e) return e;
        e = cuda_check(cudaMemsetAsync(cnt, 0, 32, st), "walk counters");
        if (e) return e;
        const uint64_t capn = 1ull << lgn;
        k_sp_fill<<<sp_grid(capn), 256, 0, st>>>(W.idx[os], capn);
        if (n) k_sp_step<<<sp_grid(n), 256, 0, st>>>(P, B, curA, n, curH, W.idx[os], W.changed, W.cap_n, cnt);
        k_sp_compact<<<sp_grid((capn + 7) / 8), 256, 0, st>>>(W.idx[os], capn, W.arr[os], W.cap_n, cnt);
        e = cuda_check(cudaGetLastError(), "walk step");
        if (!e) e = read_counters();
        if (e) return e;
        uint64_t nn = hb[3];
        const uint64_t nch = P.want_changed ? hb[1] : 0;
        const unsigned long long *jH = reinterpret_cast<const unsigned long long *>((uintptr_t)f[SW_JTAB]);
        const uint64_t jt = (uint64_t)f[SW_JTMASK] & SP_KEYMASK;
        o[5] = (int64_t)nn;
        if (jH && nch)
            k_sp_join_acc<<<sp_grid(nch), 256, 0, st>>>(W.changed, nch, jH, (int)f[SW_JLG], jt, res + i);
        const unsigned long long *nA = W.arr[os], *nH = W.idx[os];
        int nlg = lgn, ns = os;
        if (f[SW_TRUNC] >= 0) {
            if (jH && nn) k_sp_join_acc<<<sp_grid(nn), 256, 0, st>>>(nA, nn, jH, (int)f[SW_JLG], jt, res + i);
            int ts = 0;
            while (ts == os) ts++;
            const int lgt = lg_for(nn);
            e = cuda_check(cudaMemsetAsync(cnt, 0, 32, st), "walk counters");
            if (e) return e;
            k_sp_fill<<<sp_grid(1ull << lgt), 256, 0, st>>>(W.idx[ts], 1ull << lgt);
            if (nn) k_sp_build<<<sp_grid(nn), 256, 0, st>>>(nA, nn, W.idx[ts], lgt, (int)f[SW_TRUNC], W.arr[ts], cnt);
            e = cuda_check(cudaGetLastError(), "walk truncate");
            if (!e) e = read_counters();
            if (e) return e;
            nn = hb[3];
            nA = W.arr[ts];
            nH = W.idx[ts];
            nlg = lgt;
            ns = ts;
        }
        o[0] = (int64_t)nn;
        o[1] = (int64_t)nch;
        o[2] = o[3] = -1;
        o[4] = nlg;
        if (f[SW_KEEP] == 1 || (f[SW_KEEP] == 2 && nn <= SPW_KEEP_SMALL)) {
            // the kept copy gets an index of its own at load <= 1/2 (half the working index)
            const int lgk = lg_for(nn);
            const uint64_t ab = (8 * nn + 255) / 256 * 256, ib = 8ull << lgk;
            if (!arena || used + ab + ib > arena_bytes) { need[1] = (int64_t)(used + ab + ib); return i; }
            uint8_t *base = static_cast<uint8_t *>(arena);
            unsigned long long *kA = reinterpret_cast<unsigned long long *>(base + used);
            unsigned long long *kH = reinterpret_cast<unsigned long long *>(base + used + ab);
            if (nn) e = cuda_check(cudaMemcpyAsync(kA, nA, 8 * nn, cudaMemcpyDeviceToDevice, st), "keep array");
            if (e) return e;
            k_sp_fill<<<sp_grid(1ull << lgk), 256, 0, st>>>(kH, 1ull << lgk);
            if (nn) k_sp_build<<<sp_grid(nn), 256, 0, st>>>(kA, nn, kH, lgk, -1, nullptr, cnt);
            e = cuda_check(cudaGetLastError(), "keep index");
            if (e) return e;
            o[2] = (int64_t)used;
            o[3] = (int64_t)(used + ab);
            o[4] = lgk;
            used += ab + ib;
        }
        curA = nA;
        curH = nH;
        n = nn;
        lg = nlg;
        cur = ns;
    }
    return nsteps;
}

// Lookahead classes of every cut of a sparse trellis (host work, no GPU; the per-cut loop of
// cdist/sparse_dp.py:148-192 in C++).  Rows are given as sorted column positions (row_ptr /
// row_cols, CSR), columns as rows (col_ptr / col_rows), the active rows of each cut (act_ptr /
// act_rows), each row's first and last position and slot, the target row L.  For cut c the
// relevant rows are the active ones (plus L while it lies wholly on the remaining side); row r gets
// weight Q / (max over the remaining columns j containing r of |supp(j) ∩ relevant|); rows are
// grouped into classes of equal weight (masks of slots, weights ascending), L's weight is `extra`.
// Output per cut: ncls[c], masks / weights [c][maxc], extra[c].  Returns 0, or -4 if a cut has
// more than maxc classes.
int tg_sp_bound_data_wide(int N, int nrows, const int64_t *row_ptr, const int32_t *row_cols, const int64_t *col_ptr,
                          const int32_t *col_rows, const int64_t *act_ptr, const int32_t *act_rows,
                          const int32_t *row_start, const int32_t *row_end, const int32_t *slot, int L, int forward,
                          int maxc, int words, int32_t *ncls, uint64_t *masks, int64_t *weights, int64_t *extra) {
    if (N < 0 || nrows <= 0 || !row_ptr || !col_ptr || !act_ptr || !ncls || !masks || !weights || !extra || maxc < 1 ||
        words < 1)
        return set_error(TG_ERR_ARG, "bad bound data");
    for (int r = 0; r < nrows; r++)
        if (slot[r] < 0 || slot[r] >= 64 * words) return set_error(TG_ERR_ARG, "row slot beyond the mask words");
    std::vector<char> inrel(nrows, 0);
    std::vector<int> rel;
    // weight classes: (weight in 1/Q units, first row of the class); a row joins its class's mask
    std::vector<std::pair<int64_t, std::vector<uint64_t>>> cls;
    for (int c = 0; c <= N; c++) {
        rel.assign(act_rows + act_ptr[c], act_rows + act_ptr[c + 1]);
        const bool lone = forward ? row_start[L] >= c : row_end[L] < c;
        if (lone && std::find(rel.begin(), rel.end(), L) == rel.end()) rel.push_back(L);
        ncls[c] = 0;
        extra[c] = 0;
        if (rel.empty()) continue;
        int lo, hi;
        if (forward) {
            lo = c;
            hi = 0;
            for (int r : rel) hi = std::max(hi, row_end[r] + 1);
        } else {
            lo = N;
            for (int r : rel) lo = std::min(lo, row_start[r]);
            hi = c;
        }
        for (int r : rel) inrel[r] = 1;
        cls.clear();
        for (int r : rel) {
            const int32_t *b = row_cols + row_ptr[r], *e = row_cols + row_ptr[r + 1];
            int worst = 0;
            for (const int32_t *q = std::lower_bound(b, e, lo); q < e && *q < hi; q++) {
                int cnt = 0;
                for (int64_t k = col_ptr[*q]; k < col_ptr[*q + 1]; k++) cnt += inrel[col_rows[k]];
                worst = std::max(worst, cnt);
            }
            if (worst < 1) {
                for (int r2 : rel) inrel[r2] = 0;
                return set_error(TG_ERR_STATE, "a relevant row without a remaining column");
            }
            const int64_t wr = SP_QW / worst;
            if (lone && r == L) { extra[c] = wr; continue; }
            size_t k = 0;
            while (k < cls.size() && cls[k].first != wr) k++;
            if (k == cls.size()) cls.push_back({wr, std::vector<uint64_t>(words, 0ull)});
            cls[k].second[slot[r] >> 6] |= 1ull << (slot[r] & 63);
        }
        for (int r : rel) inrel[r] = 0;
        if ((int)cls.size() > maxc) return set_error(TG_ERR_TOO_BIG, "more lookahead classes than the output holds");
        std::sort(cls.begin(), cls.end());
        ncls[c] = (int32_t)cls.size();
        for (size_t k = 0; k < cls.size(); k++) {
            weights[(size_t)c * maxc + k] = cls[k].first;
            for (int w = 0; w < words; w++) masks[((size_t)c * maxc + k) * words + w] = cls[k].second[w];
        }
    }
    return TG_OK;
}

int tg_sp_bound_data(int N, int nrows, const int64_t *row_ptr, const int32_t *row_cols, const int64_t *col_ptr,
                     const int32_t *col_rows, const int64_t *act_ptr, const int32_t *act_rows, const int32_t *row_start,
                     const int32_t *row_end, const int32_t *slot, int L, int forward, int maxc, int32_t *ncls,
                     uint64_t *masks, int64_t *weights, int64_t *extra) {
    return tg_sp_bound_data_wide(N, nrows, row_ptr, row_cols, col_ptr, col_rows, act_ptr, act_rows, row_start, row_end,
                                 slot, L, forward, maxc, 1, ncls, masks, weights, extra);
}

// GF(2) rank of the first i columns of `order` for i = 0..ncols (host work, no GPU; the rank
// profile of cdist/trellis.py:20-36 with word-parallel bitsets).  Columns as rows (col_ptr /
// col_rows CSR over nrows rows); out: int32[ncols + 1].
int tg_rank_profile(int ncols, int nrows, const int64_t *col_ptr, const int32_t *col_rows, const int32_t *order,
                    int32_t *out) {
    if (ncols < 0 || nrows < 0 || !col_ptr || !order || !out) return set_error(TG_ERR_ARG, "bad rank profile");
    const int W = (nrows + 63) / 64;
    std::vector<uint64_t> piv((size_t)std::max(nrows, 1) * std::max(W, 1), 0);   // pivot vector by its top bit
    std::vector<char> has(std::max(nrows, 1), 0);
    std::vector<uint64_t> v(std::max(W, 1));
    int rank = 0;
    out[0] = 0;
    for (int i = 0; i < ncols; i++) {
        std::fill(v.begin(), v.end(), 0ull);
        const int j = order[i];
        for (int64_t k = col_ptr[j]; k < col_ptr[j + 1]; k++) v[col_rows[k] >> 6] ^= 1ull << (col_rows[k] & 63);
        int top_word = W - 1;
        while (true) {
            while (top_word >= 0 && v[top_word] == 0) top_word--;
            if (top_word < 0) break;
            const int top = top_word * 64 + 63 - __builtin_clzll(v[top_word]);
            if (!has[top]) {
                has[top] = 1;
                std::copy(v.begin(), v.end(), piv.begin() + (size_t)top * W);
                rank++;
                break;
            }
            const uint64_t *p = piv.data() + (size_t)top * W;
            for (int w = 0; w <= top_word; w++) v[w] ^= p[w];
        }
        out[i + 1] = rank;
    }
    return TG_OK;
}

// Index (2^lg slots, cleared by the call) of an array of distinct packed states.  below >= 0:
// only states with value < below are indexed, and copied to `kept` (room for n) when it is given.
int tg_sp_build(const void *A, uint64_t n, void *H, int lg, int below, void *kept, void *counters, void *stream) {
    if (lg < 1 || lg > 40 || !H || !counters || (n && !A)) return set_error(TG_ERR_ARG, "bad index build");
    cudaStream_t st = (cudaStream_t)stream;
    int e = cuda_check(cudaMemsetAsync(counters, 0, 4 * sizeof(unsigned long long), st), "counters");
    if (e) return e;
    const uint64_t cap = 1ull << lg;
    k_sp_fill<<<sp_grid(cap), 256, 0, st>>>((unsigned long long *)H, cap);
    if (n) k_sp_build<<<sp_grid(n), 256, 0, st>>>((const unsigned long long *)A, n, (unsigned long long *)H, lg, below,
                                                 (unsigned long long *)kept, (unsigned long long *)counters);
    return cuda_check(cudaGetLastError(), "index build");
}

// Join of nf changed states F against a backward index; result (device, 1 x uint64) is set to
// all ones by the call and holds the packed minimum afterwards (all ones: no pair).
int tg_sp_join(const void *F, uint64_t nf, const void *Hb, int lgb, uint64_t tmask, void *result, void *stream) {
    if (!result || (nf && (!F || !Hb))) return set_error(TG_ERR_ARG, "bad join");
    cudaStream_t st = (cudaStream_t)stream;
    int e = cuda_check(cudaMemsetAsync(result, 0xFF, sizeof(unsigned long long), st), "join init");
    if (e) return e;
    if (nf) k_sp_join<<<sp_grid(nf), 256, 0, st>>>((const unsigned long long *)F, nf, (const unsigned long long *)Hb, lgb,
                                                  tmask & SP_KEYMASK, (unsigned long long *)result);
    return cuda_check(cudaGetLastError(), "join");
}

// Values (255 = absent) of n keys in an index.
int tg_sp_lookup(const void *H, int lg, const void *keys, uint64_t n, void *vals, void *stream) {
    if (!H || (n && (!keys || !vals))) return set_error(TG_ERR_ARG, "bad lookup");
    if (n) k_sp_lookup<<<sp_grid(n), 256, 0, (cudaStream_t)stream>>>((const unsigned long long *)H, lg,
                                                                     (const unsigned long long *)keys, n, (uint8_t *)vals);
    return cuda_check(cudaGetLastError(), "lookup");
}

// Value histogram of an array into hist (device, 256 x uint64, zeroed by the call).
int tg_sp_hist(const void *A, uint64_t n, void *hist, void *stream) {
    cudaStream_t st = (cudaStream_t)stream;
    int e = cuda_check(cudaMemsetAsync(hist, 0, 256 * sizeof(unsigned long long), st), "hist clear");
    if (e) return e;
    if (n) k_sp_hist<<<sp_grid(n), 256, 0, st>>>((const unsigned long long *)A, n, (unsigned long long *)hist);
    return cuda_check(cudaGetLastError(), "hist");
}

}  // extern "C"
