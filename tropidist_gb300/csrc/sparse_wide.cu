// Sparse (weight-truncated) Rank DP on device tables whose states are wider than one machine word.
//
// The reference packs a state into one uint64 (at most 56 row slots in C, 64 in numpy,
// cdist/sparse_dp.c:3-4, cdist/sparse_dp.py:97-98) and refuses wider trellises; a circuit-style
// detector error model of 150 checks per round needs about 260 slots.  Here a state is W uint64
// words (W <= 8: up to 512 slots) and a table is
//   keys  uint64 [W][cap]  (word-major: word w of state i at w * cap + i, coalesced per word),
//   vals  uint8  [cap],
//   index uint64 [2^lg]    open addressing by a hash of the W words, slot = value << 56 | state;
//                          empty = all ones; the key itself is read from the key array.
// One column step (the rule of cdist/sparse_dp.py:338-403 with a column weight w) is two kernels:
//   emit     for every old state i: the state itself (closing-row filter, bits cleared, cap and
//            lookahead) at staging position 2i, and its candidate key ^ upd with value v + w
//            (from v < cap, same filters) at 2i + 1; each emitted key is written to the staging
//            array and then inserted into a staging index with an atomic minimum on the slot word,
//            comparing keys against the staging array (the writer fences between its key stores
//            and its compare-and-swap, the reader fences between the atomic and its key loads);
//   compact  every occupied staging slot (the least value per key) goes to the new table when its
//            value is below keep_below, and with its own index built in the same pass (the keys are
//            distinct); a slot won by a candidate whose value is below the old table's value of the
//            same key (looked up in the OLD index, the closing bits restored) is a changed state.
// The result is a set of per-key minima whatever the thread order, so the tables equal the
// reference rule's tables as sets.  Every probe loop is bounded by the index capacity and raises
// an error flag when it runs out.
#include "tg_common.cuh"
#include "tg_capi.h"

#include <algorithm>
#include <cstring>

namespace tg {

#define SPW_EMPTY 0xFFFFFFFFFFFFFFFFull
#define SPW_IDX ((1ull << 40) - 1)
#define SPW_QW 720720ll
#define SPW_MAXW 8
#define SPW_MAXCLS 32
#define SPW_PER 4               // slots per thread in a tile of a compaction or a filter

struct WideBound {
    int on, ncls, K, pad;
    int64_t extra;
    uint64_t tmask[SPW_MAXW];
    uint64_t mask[SPW_MAXCLS][SPW_MAXW];
    int64_t w[SPW_MAXCLS];
};

struct WideStep {
    uint64_t upd[SPW_MAXW], sel_mask[SPW_MAXW], sel_bits[SPW_MAXW];
    int cap, keep_below, w, want_changed;
};

// SplitMix64 finalizer (Steele, Lea, Flood 2014) over the words, each mixed with its position
__device__ __forceinline__ uint64_t spw_mix(uint64_t x) {
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ull;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebull;
    x ^= x >> 31;
    return x;
}

template <int W>
__device__ __forceinline__ uint32_t spw_slot(const uint64_t (&k)[W], int lg) {
    uint64_t h = 0x9E3779B97F4A7C15ull;
#pragma unroll
    for (int w = 0; w < W; w++) h = spw_mix(h ^ (k[w] + 0x632BE59BD9B4E019ull * (uint64_t)(w + 1)));
    return (uint32_t)(h >> (64 - lg));
}

template <int W>
__device__ __forceinline__ void spw_load(const uint64_t *keys, uint64_t stride, uint64_t i, uint64_t (&k)[W]) {
#pragma unroll
    for (int w = 0; w < W; w++) k[w] = keys[(uint64_t)w * stride + i];
}

// key words written by other threads of the same launch: read through L2
template <int W>
__device__ __forceinline__ bool spw_equal_cg(const uint64_t *keys, uint64_t stride, uint64_t i, const uint64_t (&k)[W]) {
    bool eq = true;
#pragma unroll
    for (int w = 0; w < W; w++) eq = eq && __ldcg(keys + (uint64_t)w * stride + i) == k[w];
    return eq;
}

// ceil((extra + sum_c w_c * |(key ^ tmask) & mask_c|) / QW)   (cdist/sparse_dp.py:208-217)
template <int W>
__device__ __forceinline__ bool spw_keep(const WideBound &b, const uint64_t (&k)[W], uint32_t v) {
    if (!b.on) return true;
    int64_t tot = b.extra;
    for (int c = 0; c < b.ncls; c++) {
        int cnt = 0;
#pragma unroll
        for (int w = 0; w < W; w++) cnt += __popcll((k[w] ^ b.tmask[w]) & b.mask[c][w]);
        tot += b.w[c] * (int64_t)cnt;
    }
    return (int64_t)v + (tot + SPW_QW - 1) / SPW_QW <= (int64_t)b.K;
}

// value of key in a table's index (255 when absent)
template <int W>
__device__ __forceinline__ uint32_t spw_lookup(const unsigned long long *H, int lg, const uint64_t *keys,
                                               uint64_t stride, const uint64_t (&k)[W]) {
    if (!H) return 255u;
    const uint32_t mask = (1u << lg) - 1u;
    uint32_t s = spw_slot<W>(k, lg);
    for (uint32_t probe = 0; probe <= mask; probe++) {
        const unsigned long long cur = __ldcg(H + s);
        if (cur == SPW_EMPTY) return 255u;
        if (spw_equal_cg<W>(keys, stride, cur & SPW_IDX, k)) return (uint32_t)(cur >> 56);
        s = (s + 1) & mask;
    }
    return 255u;
}

// The threads that share a range: the whole grid (separate launches per phase) or one block (a
// walk of small tables in one launch).  Element loops step by `step` from `first`; tile loops (block
// collectives inside) step by `tstep` from `tile0` and add threadIdx.x.
struct Lanes {
    uint64_t first, step, tile0, tstep;
};
__device__ __forceinline__ Lanes grid_lanes() {
    const uint64_t nt = (uint64_t)gridDim.x * blockDim.x, b0 = (uint64_t)blockIdx.x * blockDim.x;
    return Lanes{b0 + threadIdx.x, nt, b0, nt};
}
__device__ __forceinline__ Lanes block_lanes() { return Lanes{threadIdx.x, blockDim.x, 0, blockDim.x}; }

// staging: write the key, then insert value << 56 | e keeping the least word per key (BLK: all
// writers and readers are threads of one block)
template <int W, bool BLK>
__device__ __forceinline__ void spw_emit(uint64_t *ek, uint64_t estride, uint8_t *ev, unsigned long long *H, int lg,
                                         uint64_t e, const uint64_t (&k)[W], uint32_t v, unsigned long long *err) {
#pragma unroll
    for (int w = 0; w < W; w++) __stcg(ek + (uint64_t)w * estride + e, k[w]);
    ev[e] = (uint8_t)v;
    if (BLK) __threadfence_block();
    else __threadfence();
    const unsigned long long word = ((unsigned long long)v << 56) | e;
    const uint32_t mask = (1u << lg) - 1u;
    uint32_t s = spw_slot<W>(k, lg);
    for (uint32_t probe = 0; probe <= mask; probe++) {
        unsigned long long cur = atomicCAS(H + s, SPW_EMPTY, word);
        if (cur == SPW_EMPTY) return;
        if (BLK) __threadfence_block();
        else __threadfence();
        if (spw_equal_cg<W>(ek, estride, cur & SPW_IDX, k)) {
            atomicMin(H + s, word);
            return;
        }
        s = (s + 1) & mask;
    }
    atomicOr(err, 1ull);
}

__device__ __forceinline__ void spw_fill_body(const Lanes &L, unsigned long long *H, uint64_t m) {
    for (uint64_t i = L.first; i < m; i += L.step) H[i] = SPW_EMPTY;
}

__global__ void k_spw_fill(unsigned long long *H, uint64_t n) { spw_fill_body(grid_lanes(), H, n); }

// n_dev (or null): the table's size on the device, clamped to n (its capacity)
__device__ __forceinline__ uint64_t spw_count(const unsigned long long *n_dev, uint64_t n) {
    if (!n_dev) return n;
    const uint64_t d = __ldcg(n_dev);
    return d < n ? d : n;
}

// every old state and its candidate through the column into the staging index
template <int W, bool BLK>
__device__ __forceinline__ void spw_emit_body(const Lanes &L, const uint64_t *__restrict__ keys,
                                              const uint8_t *__restrict__ vals, uint64_t n, uint64_t stride,
                                              uint64_t *ek, uint8_t *ev, uint64_t estride, unsigned long long *H,
                                              int lg, const WideStep &P, const WideBound &B,
                                              unsigned long long *counters) {
    for (uint64_t i = L.first; i < n; i += L.step) {
        uint64_t k[W];
        spw_load<W>(keys, stride, i, k);
        const uint32_t v = vals[i];
        // the old state
        bool pass = true;
#pragma unroll
        for (int w = 0; w < W; w++) pass = pass && (k[w] & P.sel_mask[w]) == P.sel_bits[w];
        if (pass) {
            uint64_t c[W];
#pragma unroll
            for (int w = 0; w < W; w++) c[w] = k[w] & ~P.sel_mask[w];
            if ((int)v <= P.cap && spw_keep<W>(B, c, v))
                spw_emit<W, BLK>(ek, estride, ev, H, lg, 2 * i, c, v, counters + 2);
        }
        // its candidate
        if ((int)v < P.cap && (int)v + P.w <= P.cap) {
            uint64_t c[W];
            bool cpass = true, any = false;
#pragma unroll
            for (int w = 0; w < W; w++) {
                c[w] = k[w] ^ P.upd[w];
                any = any || P.upd[w] != 0;
                cpass = cpass && (c[w] & P.sel_mask[w]) == P.sel_bits[w];
                c[w] &= ~P.sel_mask[w];
            }
            const uint32_t cv = v + (uint32_t)P.w;
            if (any && cpass && spw_keep<W>(B, c, cv))
                spw_emit<W, BLK>(ek, estride, ev, H, lg, 2 * i + 1, c, cv, counters + 2);
        }
    }
}

template <int W>
__global__ void k_spw_emit(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ vals, uint64_t n,
                           uint64_t stride, uint64_t *ek, uint8_t *ev, uint64_t estride, unsigned long long *H, int lg,
                           const WideStep P, const WideBound B, unsigned long long *counters,
                           const unsigned long long *n_dev = nullptr, const unsigned long long *lg_dev = nullptr,
                           const unsigned long long *abort = nullptr) {
    n = (abort && *abort) ? 0 : spw_count(n_dev, n);
    if (lg_dev) lg = (int)*lg_dev;
    spw_emit_body<W, false>(grid_lanes(), keys, vals, n, stride, ek, ev, estride, H, lg, P, B, counters);
}

// new table (keys, vals, index lg2) from the staging index; changed states from candidate slots.
// Tiles of blockDim slots: output positions are claimed once per block and tile.
template <int W>
__device__ __forceinline__ void spw_compact_body(const Lanes &L, const unsigned long long *__restrict__ H,
                                                 uint64_t hcap, const uint64_t *__restrict__ ek, uint64_t estride,
                                                 uint64_t *nk, uint8_t *nv, uint64_t ncap, unsigned long long *H2,
                                                 int lg2, uint64_t *ck, uint8_t *cv, uint64_t ccap,
                                                 const unsigned long long *Hold, int lg_old, const uint64_t *okeys,
                                                 uint64_t ostride, const WideStep &P, unsigned long long *counters) {
    // tiles of SPW_PER slots per thread: output positions are claimed once per block and tile;
    // the key words of a slot are read when its flags are decided and again when it is written
    unsigned phase = 0;
    const uint32_t mask2 = (1u << lg2) - 1u;
    for (uint64_t t0 = L.tile0 * SPW_PER; t0 < hcap; t0 += L.tstep * SPW_PER) {
        unsigned long long cw[SPW_PER];
        unsigned kmask = 0, cmask = 0;
#pragma unroll
        for (int q = 0; q < SPW_PER; q++) {
            const uint64_t s = t0 + (uint64_t)q * blockDim.x + threadIdx.x;
            const unsigned long long cur = s < hcap ? __ldcg(H + s) : SPW_EMPTY;
            cw[q] = cur;
            if (cur == SPW_EMPTY) continue;
            const uint64_t e = cur & SPW_IDX;
            const uint32_t v = (uint32_t)(cur >> 56);
            if (!(P.keep_below >= 0 && (int)v >= P.keep_below)) kmask |= 1u << q;
            if (P.want_changed && (e & 1ull)) {
                // a candidate won: changed unless the old table had this key (closing bits
                // restored) with a value <= v
                uint64_t o[W];
                spw_load<W>(ek, estride, e, o);
#pragma unroll
                for (int w = 0; w < W; w++) o[w] |= P.sel_bits[w];
                if (v < spw_lookup<W>(Hold, lg_old, okeys, ostride, o)) cmask |= 1u << q;
            }
        }
        unsigned long long j, jc;
        block_claim2_n(phase, counters, __popc(kmask), P.want_changed ? counters + 1 : nullptr, __popc(cmask), j, jc);
#pragma unroll
        for (int q = 0; q < SPW_PER; q++) {
            if (!(((kmask | cmask) >> q) & 1u)) continue;
            const uint64_t e = cw[q] & SPW_IDX;
            const uint32_t v = (uint32_t)(cw[q] >> 56);
            uint64_t k[W];
            spw_load<W>(ek, estride, e, k);
            if ((cmask >> q) & 1u) {
                if (jc < ccap) {
#pragma unroll
                    for (int w = 0; w < W; w++) ck[(uint64_t)w * ccap + jc] = k[w];
                    cv[jc] = (uint8_t)v;
                } else {
                    atomicOr(counters + 2, 2ull);
                }
                jc++;
            }
            if (!((kmask >> q) & 1u)) continue;
            if (j >= ncap) {
                atomicOr(counters + 2, 4ull);
                j++;
                continue;
            }
#pragma unroll
            for (int w = 0; w < W; w++) nk[(uint64_t)w * ncap + j] = k[w];
            nv[j] = (uint8_t)v;
            // the keys are distinct: claim the first empty slot
            uint32_t t = spw_slot<W>(k, lg2);
            uint32_t probe = 0;
            for (; probe <= mask2; probe++) {
                if (atomicCAS(H2 + t, SPW_EMPTY, ((unsigned long long)v << 56) | j) == SPW_EMPTY) break;
                t = (t + 1) & mask2;
            }
            if (probe > mask2) atomicOr(counters + 2, 1ull);
            j++;
        }
    }
}

template <int W>
__global__ void k_spw_compact(const unsigned long long *__restrict__ H, uint64_t hcap, const uint64_t *__restrict__ ek,
                              uint64_t estride, uint64_t *nk, uint8_t *nv, uint64_t ncap, unsigned long long *H2,
                              int lg2, uint64_t *ck, uint8_t *cv, uint64_t ccap, const unsigned long long *Hold,
                              int lg_old, const uint64_t *okeys, uint64_t ostride, const WideStep P,
                              unsigned long long *counters, const unsigned long long *lg_dev = nullptr,
                              const unsigned long long *lg_old_dev = nullptr) {
    if (lg_dev) {
        lg2 = (int)*lg_dev;
        hcap = 1ull << lg2;
    }
    if (lg_old_dev) lg_old = (int)*lg_old_dev;
    spw_compact_body<W>(grid_lanes(), H, hcap, ek, estride, nk, nv, ncap, H2, lg2, ck, cv, ccap, Hold, lg_old, okeys,
                        ostride, P, counters);
}

// a table's states with value < below (all when below < 0) into (nk, nv) with their own index
template <int W>
__device__ __forceinline__ void spw_filter_body(const Lanes &L, const uint64_t *__restrict__ keys,
                                                const uint8_t *__restrict__ vals, uint64_t n, uint64_t stride,
                                                int below, uint64_t *nk, uint8_t *nv, uint64_t ncap,
                                                unsigned long long *H2, int lg2, unsigned long long *counters) {
    unsigned phase = 0;
    const uint32_t mask2 = (1u << lg2) - 1u;
    for (uint64_t t0 = L.tile0 * SPW_PER; t0 < n; t0 += L.tstep * SPW_PER) {
        unsigned wmask = 0;
#pragma unroll
        for (int q = 0; q < SPW_PER; q++) {
            const uint64_t i = t0 + (uint64_t)q * blockDim.x + threadIdx.x;
            if (i < n && !(below >= 0 && (int)vals[i] >= below)) wmask |= 1u << q;
        }
        unsigned long long j, unused;
        block_claim2_n(phase, counters, __popc(wmask), nullptr, 0u, j, unused);
#pragma unroll
        for (int q = 0; q < SPW_PER; q++) {
            if (!((wmask >> q) & 1u)) continue;
            const uint64_t i = t0 + (uint64_t)q * blockDim.x + threadIdx.x;
            if (j >= ncap) {
                atomicOr(counters + 2, 4ull);
                j++;
                continue;
            }
            const uint32_t v = vals[i];
            uint64_t k[W];
            spw_load<W>(keys, stride, i, k);
#pragma unroll
            for (int w = 0; w < W; w++) nk[(uint64_t)w * ncap + j] = k[w];
            nv[j] = (uint8_t)v;
            uint32_t t = spw_slot<W>(k, lg2);
            uint32_t probe = 0;
            for (; probe <= mask2; probe++) {
                if (atomicCAS(H2 + t, SPW_EMPTY, ((unsigned long long)v << 56) | j) == SPW_EMPTY) break;
                t = (t + 1) & mask2;
            }
            if (probe > mask2) atomicOr(counters + 2, 1ull);
            j++;
        }
    }
}

template <int W>
__global__ void k_spw_filter(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ vals, uint64_t n,
                             uint64_t stride, int below, uint64_t *nk, uint8_t *nv, uint64_t ncap,
                             unsigned long long *H2, int lg2, unsigned long long *counters,
                             const unsigned long long *n_dev = nullptr, const unsigned long long *lg_dev = nullptr) {
    n = spw_count(n_dev, n);
    if (lg_dev) lg2 = (int)*lg_dev;
    spw_filter_body<W>(grid_lanes(), keys, vals, n, stride, below, nk, nv, ncap, H2, lg2, counters);
}

// least f.value + b.value over changed f and backward b with key(b) = key(f) ^ tmask:
// result = min(total << 40 | tag | f)
template <int W>
__device__ __forceinline__ void spw_join_body(const Lanes &L, const uint64_t *__restrict__ fk,
                                              const uint8_t *__restrict__ fv, uint64_t nf, uint64_t fstride,
                                              const unsigned long long *__restrict__ Hb, int lgb,
                                              const uint64_t *__restrict__ bk, uint64_t bstride,
                                              const uint64_t *tmask, unsigned long long *result, uint64_t tag) {
    for (uint64_t i = L.first; i < nf; i += L.step) {
        uint64_t q[W];
        spw_load<W>(fk, fstride, i, q);
#pragma unroll
        for (int w = 0; w < W; w++) q[w] ^= tmask[w];
        const uint32_t bv = spw_lookup<W>(Hb, lgb, bk, bstride, q);
        if (bv == 255u) continue;
        atomicMin(result, ((unsigned long long)(fv[i] + bv) << 40) | tag | i);
    }
}

template <int W>
__global__ void k_spw_join(const uint64_t *__restrict__ fk, const uint8_t *__restrict__ fv, uint64_t nf,
                           uint64_t fstride, const unsigned long long *__restrict__ Hb, int lgb,
                           const uint64_t *__restrict__ bk, uint64_t bstride, const WideBound T,
                           unsigned long long *result, const unsigned long long *n_dev = nullptr,
                           uint64_t tag = 0) {
    nf = spw_count(n_dev, nf);
    spw_join_body<W>(grid_lanes(), fk, fv, nf, fstride, Hb, lgb, bk, bstride, T.tmask, result, tag);
}

template <int W>
__global__ void k_spw_lookup(const unsigned long long *__restrict__ H, int lg, const uint64_t *__restrict__ keys,
                             uint64_t stride, const uint64_t *__restrict__ q, uint64_t m, uint8_t *out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t k[W];
        spw_load<W>(q, m, i, k);
        out[i] = (uint8_t)spw_lookup<W>(H, lg, keys, stride, k);
    }
}

// ---- kernels of a walk: the table sizes and index widths stay on the device between steps
#define SPW_TAG (1ull << 39)          // join result from a whole table (not the changed list)
#define SPW_KEEP_SMALL 1024           // keep mode 2: only tables of at most this many states

__device__ __forceinline__ int spw_lg_dev(uint64_t n) {         // index bits for n states at load <= 1/2
    int lg = 6;
    while ((1ull << lg) < 2 * n) lg++;
    return lg;
}

// place of a kept table in the arena: rec = [n, offset, flags, lg, stride, -, -, -]; flags 8: no
// room (used still grows by the bytes it needed), 16: not kept (keep mode 2 and a large table)
__device__ __forceinline__ uint64_t spw_keep_bytes(int W, uint64_t stride, int lg) {
    return ((uint64_t)W * stride * 8 + (stride + 255) / 256 * 256 + (8ull << lg) + 255) / 256 * 256;
}

__device__ __forceinline__ void spw_keep_place(uint64_t n, int W, int mode, unsigned long long *rec,
                                               unsigned long long *used, uint64_t arena_bytes) {
    if (mode == 2 && n > SPW_KEEP_SMALL) {
        rec[2] = 16;
        return;
    }
    const uint64_t stride = n < 1 ? 1 : n;
    const int lg = spw_lg_dev(n);
    const uint64_t b = spw_keep_bytes(W, stride, lg), off = *used;
    *used = off + b;
    rec[3] = (unsigned long long)lg;
    rec[4] = stride;
    if (off + b > arena_bytes) {
        rec[2] = 8;
        return;
    }
    rec[1] = off;
}

__global__ void k_spw_keep_alloc(const unsigned long long *n_dev, uint64_t ncap, int W, int mode,
                                 unsigned long long *rec, unsigned long long *used, uint64_t arena_bytes) {
    if (threadIdx.x || blockIdx.x) return;
    spw_keep_place(spw_count(n_dev, ncap), W, mode, rec, used, arena_bytes);
}

__device__ __forceinline__ unsigned long long *spw_keep_index(uint8_t *arena, const unsigned long long *rec, int W) {
    const uint64_t stride = rec[4];
    return reinterpret_cast<unsigned long long *>(arena + rec[1] + (uint64_t)W * stride * 8 + (stride + 255) / 256 * 256);
}

__global__ void k_spw_keep_fill(uint8_t *arena, const unsigned long long *rec, int W) {
    if (rec[2] & 24ull) return;
    spw_fill_body(grid_lanes(), spw_keep_index(arena, rec, W), 1ull << rec[3]);
}

template <int W>
__device__ __forceinline__ void spw_keep_body(const Lanes &L, const uint64_t *__restrict__ keys,
                                              const uint8_t *__restrict__ vals, uint64_t n, uint64_t stride,
                                              uint8_t *arena, unsigned long long *rec) {
    const uint64_t ks = rec[4];
    uint64_t *nk = reinterpret_cast<uint64_t *>(arena + rec[1]);
    uint8_t *nv = arena + rec[1] + (uint64_t)W * ks * 8;
    spw_filter_body<W>(L, keys, vals, n, stride, -1, nk, nv, ks, spw_keep_index(arena, rec, W), (int)rec[3], rec);
}

template <int W>
__global__ void k_spw_keep(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ vals, uint64_t stride,
                           const unsigned long long *n_dev, uint8_t *arena, unsigned long long *rec) {
    if (rec[2] & 24ull) return;
    spw_keep_body<W>(grid_lanes(), keys, vals, spw_count(n_dev, stride), stride, arena, rec);
}

// the forward state (key words and value) behind a step's join result, for the host
template <int W>
__device__ __forceinline__ void spw_capture_one(const unsigned long long *result, const uint64_t *ck,
                                                const uint8_t *cv, const uint64_t *tk, const uint8_t *tv,
                                                uint64_t stride, uint64_t *resk, uint8_t *resv) {
    const unsigned long long r = *result;
    if (r == SPW_EMPTY) return;
    const uint64_t i = r & (SPW_TAG - 1);
    const uint64_t *k = (r & SPW_TAG) ? tk : ck;
    const uint8_t *v = (r & SPW_TAG) ? tv : cv;
#pragma unroll
    for (int w = 0; w < W; w++) resk[w] = k[(uint64_t)w * stride + i];
    *resv = v[i];
}

template <int W>
__global__ void k_spw_capture(const unsigned long long *result, const uint64_t *ck, const uint8_t *cv,
                              const uint64_t *tk, const uint8_t *tv, uint64_t stride, uint64_t *resk, uint8_t *resv) {
    if (threadIdx.x || blockIdx.x) return;
    spw_capture_one<W>(result, ck, cv, tk, tv, stride, resk, resv);
}

// fill the index (or two) of 2^lg slots, lg = index bits for mult * n states; *lg_out = lg.  Once a
// step has raised a flag (prev: its counter block) the walk is void: *abort is set and the later
// steps run on empty tables (the host runs the leg again with more room).  With cap_res, thread 0
// first captures the previous step's join result (its changed list and table are still intact).
template <int W>
__global__ void k_spw_fill_dyn(const unsigned long long *n_dev, uint64_t ncap, int mult, unsigned long long *lg_out,
                               unsigned long long *H1, unsigned long long *H2, const unsigned long long *prev,
                               unsigned long long *abort, const unsigned long long *cap_res = nullptr,
                               const uint64_t *cap_ck = nullptr, const uint8_t *cap_cv = nullptr,
                               const uint64_t *cap_tk = nullptr, const uint8_t *cap_tv = nullptr,
                               uint64_t cap_stride = 0, uint64_t *cap_k = nullptr, uint8_t *cap_v = nullptr) {
    if (cap_res && blockIdx.x == 0 && threadIdx.x == 0)
        spw_capture_one<W>(cap_res, cap_ck, cap_cv, cap_tk, cap_tv, cap_stride, cap_k, cap_v);
    const bool bad = *abort || (prev && ((prev[2] | prev[6]) & 7ull));
    if (bad && blockIdx.x == 0 && threadIdx.x == 0) *abort = 1;
    const int lg = spw_lg_dev(bad ? 0 : (uint64_t)mult * spw_count(n_dev, ncap));
    if (blockIdx.x == 0 && threadIdx.x == 0) *lg_out = (unsigned long long)lg;
    const uint64_t m = 1ull << lg;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x) {
        H1[i] = SPW_EMPTY;
        if (H2) H2[i] = SPW_EMPTY;
    }
}

// ---- a leg of column steps (tg_spw_walk).  Per step, int64 fields (SPW_WALK_FIELDS): cap,
// keep_below, w, trunc (< 0: none), keep (0, 1, 2: small tables only), join (a backward table to
// join), ncls, use_h, extra, join keys, join index, join index bits, join key stride; uint64 words
// [5][W]: upd, sel_mask, sel_bits, the bound's tmask, the join's tmask.
#define SPW_WALK_FIELDS 13
enum { WK_CAP, WK_KB, WK_W, WK_TRUNC, WK_KEEP, WK_JOIN, WK_NCLS, WK_USEH, WK_EXTRA, WK_JKEYS, WK_JH, WK_JLG, WK_JSTRIDE };

struct SpwRing {
    uint64_t *keys;
    uint8_t *vals;
    unsigned long long *H;
};

// Counters of a walk (uint64 blocks of 8): block 0 the start table, block i + 1 step i ([0] states,
// [1] changed, [2] flags, [3] index bits, [4] states after the cut's truncation, [5] its index
// bits, [6] its flags), block nsteps + 1 + i the keep record of step i, block 2 nsteps + 1: [0]
// arena bytes used, [1] abort, [2..4] the one-block walk's stop state.  The table before step i:
__host__ __device__ __forceinline__ int spw_prev_off(const int64_t *steps, int i, int &noff, int &lgoff) {
    const bool tr = i > 0 && steps[(size_t)SPW_WALK_FIELDS * (i - 1) + WK_TRUNC] >= 0;
    noff = tr ? 4 : 0;
    lgoff = tr ? 5 : 3;
    return 8 * i;
}

#define SPW_SMALL_THREADS 512
static uint64_t g_spw_small_limit = 512;       // the one-block walk steps tables while 2 n <= this

struct SpwSmall {
    const int64_t *steps;             // device copies of the walk's step records
    const uint64_t *words, *masks;
    const int64_t *weights;
    int maxc, K, i0, nsteps, cur;
    uint64_t cap, limit, arena_bytes;
    SpwRing ring[3], sg, ch;
    unsigned long long *cnt, *res;
    uint64_t *resk;
    uint8_t *resv, *arena;
};

// Steps i0.. of a walk in one block while the tables are small (no launch per kernel of a step):
// the same bodies as the separate kernels, with the block's barriers between them.  Stops before a
// step whose table holds more than limit / 2 states (reason 1) or after a step that raised a flag
// (reason 4, the walk is void); state: [0] next step, [1] ring slot of its table, [2] reason.
template <int W>
__global__ void __launch_bounds__(SPW_SMALL_THREADS) k_spw_walk_small(const __grid_constant__ SpwSmall S) {
    __shared__ WideStep P;
    __shared__ WideBound B;
    __shared__ uint64_t jt[SPW_MAXW];
    const Lanes L = block_lanes();
    const unsigned tid = threadIdx.x;
    unsigned long long *abort = S.cnt + 8ull * (2 * (uint64_t)S.nsteps + 1) + 1, *state = abort + 1;
    const uint64_t cap = S.cap;
    int cur = S.cur, i = S.i0, reason = 0;
    for (; i < S.nsteps; i++) {
        int noff, lgoff;
        const unsigned long long *pc = S.cnt + spw_prev_off(S.steps, i, noff, lgoff);
        const uint64_t n = spw_count(pc + noff, cap);
        const int lg_old = (int)__ldcg(pc + lgoff);
        if (__ldcg(abort)) { reason = 4; break; }
        if (2 * n > S.limit) { reason = 1; break; }
        const int64_t *f = S.steps + (size_t)SPW_WALK_FIELDS * i;
        const uint64_t *wd = S.words + (size_t)5 * W * i;
        const unsigned long long *jH = reinterpret_cast<const unsigned long long *>((uintptr_t)f[WK_JH]);
        const uint64_t *jk = reinterpret_cast<const uint64_t *>((uintptr_t)f[WK_JKEYS]);
        const bool join = f[WK_JOIN] && jH && jk;
        const int ncls = f[WK_USEH] ? (int)f[WK_NCLS] : 0;
        if (tid == 0) {
            P.cap = (int)f[WK_CAP];
            P.keep_below = (int)f[WK_KB];
            P.w = (int)f[WK_W];
            P.want_changed = f[WK_JOIN] != 0;
            B.on = (int)f[WK_USEH];
            B.ncls = ncls;
            B.K = S.K;
            B.extra = f[WK_EXTRA];
        }
        for (unsigned q = tid; q < (unsigned)W; q += blockDim.x) {
            P.upd[q] = wd[q];
            P.sel_mask[q] = wd[W + q];
            P.sel_bits[q] = wd[2 * W + q];
            B.tmask[q] = wd[3 * W + q];
            jt[q] = wd[4 * W + q];
        }
        for (unsigned c = tid; c < (unsigned)(ncls * W); c += blockDim.x)
            B.mask[c / W][c % W] = S.masks[((size_t)i * S.maxc) * W + c];
        for (unsigned c = tid; c < (unsigned)ncls; c += blockDim.x) B.w[c] = S.weights[(size_t)i * S.maxc + c];
        unsigned long long *c = S.cnt + 8ull * (i + 1);
        const int lgs = spw_lg_dev(2 * n);
        if (tid == 0) c[3] = (unsigned long long)lgs;
        const int out = (cur + 1) % 3;
        spw_fill_body(L, S.sg.H, 1ull << lgs);
        spw_fill_body(L, S.ring[out].H, 1ull << lgs);
        __syncthreads();
        spw_emit_body<W, true>(L, S.ring[cur].keys, S.ring[cur].vals, n, cap, S.sg.keys, S.sg.vals, 2 * cap, S.sg.H, lgs,
                               P, B, c);
        __syncthreads();
        spw_compact_body<W>(L, S.sg.H, 1ull << lgs, S.sg.keys, 2 * cap, S.ring[out].keys, S.ring[out].vals, cap,
                            S.ring[out].H, lgs, S.ch.keys, S.ch.vals, cap, S.ring[cur].H, lg_old, S.ring[cur].keys,
                            cap, P, c);
        __syncthreads();
        if (__ldcg(c + 2) & 7ull) { reason = 4; break; }
        const uint64_t nout = spw_count(c, cap);
        if (join)
            spw_join_body<W>(L, S.ch.keys, S.ch.vals, spw_count(c + 1, cap), cap, jH, (int)f[WK_JLG], jk,
                             (uint64_t)f[WK_JSTRIDE], jt, S.res + i, 0);
        int now = out;
        const unsigned long long *nnow = c;
        if (f[WK_TRUNC] >= 0) {
            // the cap drops at this cut: the whole table before the drop is joined too
            if (join)
                spw_join_body<W>(L, S.ring[out].keys, S.ring[out].vals, nout, cap, jH, (int)f[WK_JLG], jk,
                                 (uint64_t)f[WK_JSTRIDE], jt, S.res + i, SPW_TAG);
            const int tr = (out + 1) % 3, lgt = spw_lg_dev(nout);
            if (tid == 0) c[5] = (unsigned long long)lgt;
            spw_fill_body(L, S.ring[tr].H, 1ull << lgt);
            __syncthreads();
            spw_filter_body<W>(L, S.ring[out].keys, S.ring[out].vals, nout, cap, (int)f[WK_TRUNC], S.ring[tr].keys,
                               S.ring[tr].vals, cap, S.ring[tr].H, lgt, c + 4);
            now = tr;
            nnow = c + 4;
        }
        __syncthreads();
        if (__ldcg(c + 6) & 7ull) { reason = 4; break; }
        if (join && tid == 0)
            spw_capture_one<W>(S.res + i, S.ch.keys, S.ch.vals, S.ring[out].keys, S.ring[out].vals, cap,
                               S.resk + (size_t)i * W, S.resv + i);
        if (f[WK_KEEP]) {
            unsigned long long *rec = S.cnt + 8ull * (S.nsteps + 1 + i);
            const uint64_t nk = spw_count(nnow, cap);
            if (tid == 0) spw_keep_place(nk, W, (int)f[WK_KEEP], rec, abort - 1, S.arena ? S.arena_bytes : 0);
            __syncthreads();
            if (!(__ldcg(rec + 2) & 24ull)) {
                spw_fill_body(L, spw_keep_index(S.arena, rec, W), 1ull << __ldcg(rec + 3));
                __syncthreads();
                spw_keep_body<W>(L, S.ring[now].keys, S.ring[now].vals, nk, cap, S.arena, rec);
            }
        }
        __syncthreads();
        cur = now;
    }
    if (reason == 4 && tid == 0) *abort = 1;
    if (tid == 0) {
        state[0] = (unsigned long long)i;
        state[1] = (unsigned long long)cur;
        state[2] = (unsigned long long)reason;
    }
}

static unsigned spw_grid(uint64_t n) {
    const uint64_t b = (n + 255) / 256;
    const uint64_t cap = (uint64_t)std::max(1, sm_count()) * 8;
    return (unsigned)std::max<uint64_t>(1, std::min(b, cap));
}

static int spw_check_words(int W) {
    return (W < 1 || W > SPW_MAXW) ? set_error(TG_ERR_ARG, "state words must be 1..8") : TG_OK;
}

static int spw_bound(WideBound &B, int W, int use_h, int K, int ncls, const uint64_t *masks, const int64_t *weights,
                     int64_t extra, const uint64_t *tmask) {
    memset(&B, 0, sizeof(B));
    if (ncls > SPW_MAXCLS) return set_error(TG_ERR_TOO_BIG, "more than 32 lookahead classes");
    B.on = use_h;
    B.ncls = use_h ? ncls : 0;
    B.K = K;
    B.extra = extra;
    for (int w = 0; w < W; w++) B.tmask[w] = tmask ? tmask[w] : 0ull;
    for (int c = 0; c < B.ncls; c++) {
        B.w[c] = weights[c];
        for (int w = 0; w < W; w++) B.mask[c][w] = masks[(size_t)c * W + w];
    }
    return TG_OK;
}

template <int W>
static int spw_step_w(const uint64_t *keys, const uint8_t *vals, uint64_t n, uint64_t stride, const void *Hold,
                      int lg_old, uint64_t *ek, uint8_t *ev, uint64_t ecap, void *Hs, int lgs, uint64_t *nk,
                      uint8_t *nv, uint64_t ncap, void *Hn, int lgn, uint64_t *ck, uint8_t *cv, uint64_t ccap,
                      const WideStep &P, const WideBound &B, void *counters, cudaStream_t st) {
    unsigned long long *C = (unsigned long long *)counters;
    int e = cuda_check(cudaMemsetAsync(C, 0, 4 * sizeof(unsigned long long), st), "counters");
    if (e) return e;
    k_spw_fill<<<spw_grid(1ull << lgs), 256, 0, st>>>((unsigned long long *)Hs, 1ull << lgs);
    k_spw_fill<<<spw_grid(1ull << lgn), 256, 0, st>>>((unsigned long long *)Hn, 1ull << lgn);
    if (n) k_spw_emit<W><<<spw_grid(n), 256, 0, st>>>(keys, vals, n, stride, ek, ev, ecap, (unsigned long long *)Hs,
                                                      lgs, P, B, C);
    k_spw_compact<W><<<spw_grid(1ull << lgs), 256, 0, st>>>((const unsigned long long *)Hs, 1ull << lgs, ek, ecap, nk,
                                                            nv, ncap, (unsigned long long *)Hn, lgn, ck, cv, ccap,
                                                            (const unsigned long long *)Hold, lg_old, keys, stride, P,
                                                            C);
    return cuda_check(cudaGetLastError(), "wide step");
}

// ---- a leg of column steps in one call (no host read between steps)

static int spw_walk_lg(uint64_t n) {
    int lg = 6;
    while ((1ull << lg) < 2 * n) lg++;
    return lg;
}

// scratch: 3 ring tables and the changed list of cap states, a staging area of 2 cap, indexes of
// 2^lg(2 cap) slots; then 8 counters per step (+2) and per step a keep record; join results
static uint64_t spw_walk_layout(int W, uint64_t cap, int nsteps, uint8_t *base, SpwRing *ring, SpwRing *stage,
                                SpwRing *chg, unsigned long long **cnt, unsigned long long **res, uint64_t **resk,
                                uint8_t **resv) {
    const uint64_t ib = 8ull << spw_walk_lg(2 * cap);
    auto rnd = [](uint64_t x) { return (x + 255) / 256 * 256; };
    uint64_t off = 0;
    auto take = [&](uint64_t b) {
        uint8_t *p = base ? base + off : nullptr;
        off += rnd(b);
        return p;
    };
    for (int r = 0; r < 3; r++) {
        SpwRing t;
        t.keys = reinterpret_cast<uint64_t *>(take((uint64_t)W * cap * 8));
        t.vals = take(cap);
        t.H = reinterpret_cast<unsigned long long *>(take(ib));
        if (ring) ring[r] = t;
    }
    SpwRing sg;
    sg.keys = reinterpret_cast<uint64_t *>(take((uint64_t)W * 2 * cap * 8));
    sg.vals = take(2 * cap);
    sg.H = reinterpret_cast<unsigned long long *>(take(ib));
    SpwRing ch;
    ch.keys = reinterpret_cast<uint64_t *>(take((uint64_t)W * cap * 8));
    ch.vals = take(cap);
    ch.H = nullptr;
    unsigned long long *c = reinterpret_cast<unsigned long long *>(take(64ull * (2 * (uint64_t)nsteps + 2)));
    unsigned long long *r = reinterpret_cast<unsigned long long *>(take(8ull * nsteps + 8));
    uint64_t *rk = reinterpret_cast<uint64_t *>(take(8ull * W * nsteps + 8));
    uint8_t *rv = take((uint64_t)nsteps + 1);
    if (stage) *stage = sg;
    if (chg) *chg = ch;
    if (cnt) *cnt = c;
    if (res) *res = r;
    if (resk) *resk = rk;
    if (resv) *resv = rv;
    return off;
}

// device copies of a walk's step records (for the one-block walk), grown as needed
struct SpwRecords {
    int64_t *steps = nullptr;
    uint64_t *words = nullptr, *masks = nullptr;
    int64_t *weights = nullptr;
};

static int spw_records(int W, int nsteps, int maxc, const int64_t *steps, const uint64_t *words,
                       const uint64_t *masks, const int64_t *weights, cudaStream_t st, SpwRecords &R) {
    static thread_local uint8_t *buf = nullptr;
    static thread_local size_t buf_bytes = 0;
    auto rnd = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t bs = rnd(8ull * SPW_WALK_FIELDS * nsteps), bw = rnd(8ull * 5 * W * nsteps),
                 bm = rnd(8ull * maxc * W * nsteps), bg = rnd(8ull * maxc * nsteps), tot = bs + bw + bm + bg + 256;
    if (buf_bytes < tot) {
        if (buf) cudaFree(buf);
        buf = nullptr;
        buf_bytes = 0;
        if (cudaMalloc(&buf, tot) != cudaSuccess) {
            cudaGetLastError();
            return set_error(TG_ERR_NOMEM, "wide walk records");
        }
        buf_bytes = tot;
    }
    R.steps = reinterpret_cast<int64_t *>(buf);
    R.words = reinterpret_cast<uint64_t *>(buf + bs);
    R.masks = reinterpret_cast<uint64_t *>(buf + bs + bw);
    R.weights = reinterpret_cast<int64_t *>(buf + bs + bw + bm);
    int e = cuda_check(cudaMemcpyAsync(R.steps, steps, 8ull * SPW_WALK_FIELDS * nsteps, cudaMemcpyHostToDevice, st),
                       "walk records");
    if (!e) e = cuda_check(cudaMemcpyAsync(R.words, words, 8ull * 5 * W * nsteps, cudaMemcpyHostToDevice, st),
                           "walk records");
    if (!e) e = cuda_check(cudaMemcpyAsync(R.masks, masks, 8ull * maxc * W * nsteps, cudaMemcpyHostToDevice, st),
                           "walk records");
    if (!e) e = cuda_check(cudaMemcpyAsync(R.weights, weights, 8ull * maxc * nsteps, cudaMemcpyHostToDevice, st),
                           "walk records");
    return e;
}

#define SPW_CHUNK 32                  // steps of separate launches between two reads of the table size

// The walk: while the table is small, one launch of the one-block walk runs steps until the table
// outgrows it; larger tables take a few launches per step, SPW_CHUNK steps between reads of the
// table size (the next small stretch starts once it is back under a quarter of the limit).
template <int W>
static int spw_walk_w(int nsteps, const int64_t *steps, const uint64_t *words, const uint64_t *masks,
                      const int64_t *weights, int maxc, int K, const uint64_t *k0, const uint8_t *v0, uint64_t n0,
                      uint64_t stride0, uint8_t *scratch, uint64_t cap, uint8_t *arena, uint64_t arena_bytes,
                      unsigned long long *hb, cudaStream_t st) {
    SpwRing ring[3], sg, ch;
    unsigned long long *cnt, *res;
    uint64_t *resk;
    uint8_t *resv;
    spw_walk_layout(W, cap, nsteps, scratch, ring, &sg, &ch, &cnt, &res, &resk, &resv);
    const size_t cbytes = 64ull * (2 * (uint64_t)nsteps + 2);
    int e = cuda_check(cudaMemsetAsync(cnt, 0, cbytes, st), "walk counters");
    if (!e && nsteps) e = cuda_check(cudaMemsetAsync(res, 0xFF, 8ull * nsteps, st), "walk results");
    if (e) return e;
    for (int i = 0; i < nsteps; i++) {
        const int64_t *f = steps + (size_t)SPW_WALK_FIELDS * i;
        if (f[WK_USEH] && (f[WK_NCLS] < 0 || f[WK_NCLS] > maxc))
            return set_error(TG_ERR_ARG, "lookahead classes beyond the step's arrays");
        if (f[WK_USEH] && f[WK_NCLS] > SPW_MAXCLS) return set_error(TG_ERR_TOO_BIG, "more than 32 lookahead classes");
    }
    SpwRecords R;
    if (nsteps) e = spw_records(W, nsteps, maxc, steps, words, masks, weights, st, R);
    if (e) return e;
    unsigned long long *used = cnt + 8ull * (2 * (uint64_t)nsteps + 1), *abort = used + 1, *sstate = used + 2;
    const unsigned gc = spw_grid(cap), gi = spw_grid(1ull << spw_walk_lg(2 * cap));
    // the start table into ring slot 0
    k_spw_fill_dyn<W><<<gi, 256, 0, st>>>(nullptr, n0, 1, cnt + 3, ring[0].H, nullptr, nullptr, abort);
    if (n0)
        k_spw_filter<W><<<spw_grid(n0), 256, 0, st>>>(k0, v0, n0, stride0, -1, ring[0].keys, ring[0].vals, cap,
                                                      ring[0].H, 0, cnt, nullptr, cnt + 3);
    const uint64_t limit = std::min<uint64_t>(g_spw_small_limit, cap);
    uint64_t host_n = n0;             // the table size before step i, when known on the host
    int cur = 0, i = 0;
    while (i < nsteps) {
        if (4 * host_n <= limit) {
            SpwSmall S;
            S.steps = R.steps;
            S.words = R.words;
            S.masks = R.masks;
            S.weights = R.weights;
            S.maxc = maxc;
            S.K = K;
            S.i0 = i;
            S.nsteps = nsteps;
            S.cur = cur;
            S.cap = cap;
            S.limit = limit;
            S.arena_bytes = arena_bytes;
            for (int r = 0; r < 3; r++) S.ring[r] = ring[r];
            S.sg = sg;
            S.ch = ch;
            S.cnt = cnt;
            S.res = res;
            S.resk = resk;
            S.resv = resv;
            S.arena = arena;
            k_spw_walk_small<W><<<1, SPW_SMALL_THREADS, 0, st>>>(S);
            e = cuda_check(cudaGetLastError(), "small wide walk");
            if (!e) e = cuda_check(cudaMemcpyAsync(hb, sstate, 24, cudaMemcpyDeviceToHost, st), "walk state");
            if (!e) e = cuda_check(cudaStreamSynchronize(st), "walk sync");
            if (e) return e;
            i = (int)hb[0];
            cur = (int)hb[1];
            if (hb[2] == 4) break;    // a flag: the walk is void, the host reads why at the end
            host_n = ~0ull >> 3;      // beyond the limit until read again
            if (i >= nsteps) break;
        }
        const int stop = std::min(nsteps, i + SPW_CHUNK);
        int pend = -1, pend_out = 0;      // a join result not yet captured: its step and output slot
        for (; i < stop; i++) {
            const int64_t *f = steps + (size_t)SPW_WALK_FIELDS * i;
            const uint64_t *wd = words + (size_t)5 * W * i;
            if (f[WK_CAP] > 254 || f[WK_W] < 1 || f[WK_W] > 254) return set_error(TG_ERR_ARG, "values beyond 8 bits");
            int noff, lgoff;
            const unsigned long long *pc = cnt + spw_prev_off(steps, i, noff, lgoff);
            const unsigned long long *ncur = pc + noff, *lgcur = pc + lgoff;
            WideStep P;
            memset(&P, 0, sizeof(P));
            for (int q = 0; q < W; q++) {
                P.upd[q] = wd[q];
                P.sel_mask[q] = wd[W + q];
                P.sel_bits[q] = wd[2 * W + q];
            }
            P.cap = (int)f[WK_CAP];
            P.keep_below = (int)f[WK_KB];
            P.w = (int)f[WK_W];
            const unsigned long long *jH = reinterpret_cast<const unsigned long long *>((uintptr_t)f[WK_JH]);
            const uint64_t *jk = reinterpret_cast<const uint64_t *>((uintptr_t)f[WK_JKEYS]);
            const bool join = f[WK_JOIN] && jH && jk;
            P.want_changed = f[WK_JOIN] != 0;
            WideBound B, T;
            e = spw_bound(B, W, (int)f[WK_USEH], K, (int)f[WK_NCLS], masks + (size_t)i * maxc * W,
                          weights + (size_t)i * maxc, f[WK_EXTRA], wd + 3 * W);
            if (e) return e;
            memset(&T, 0, sizeof(T));
            for (int q = 0; q < W; q++) T.tmask[q] = wd[4 * W + q];
            unsigned long long *c = cnt + 8ull * (i + 1);
            const int out = (cur + 1) % 3;
            // staging and new index for 2 n states, then the two kernels of the step
            if (pend >= 0)
                k_spw_fill_dyn<W><<<gi, 256, 0, st>>>(ncur, cap, 2, c + 3, sg.H, ring[out].H, pc, abort, res + pend,
                                                      ch.keys, ch.vals, ring[pend_out].keys, ring[pend_out].vals, cap,
                                                      resk + (size_t)pend * W, resv + pend);
            else
                k_spw_fill_dyn<W><<<gi, 256, 0, st>>>(ncur, cap, 2, c + 3, sg.H, ring[out].H, pc, abort);
            pend = -1;
            k_spw_emit<W><<<gc, 256, 0, st>>>(ring[cur].keys, ring[cur].vals, cap, cap, sg.keys, sg.vals, 2 * cap,
                                              sg.H, 0, P, B, c, ncur, c + 3, abort);
            k_spw_compact<W><<<gi, 256, 0, st>>>(sg.H, 0, sg.keys, 2 * cap, ring[out].keys, ring[out].vals, cap,
                                                 ring[out].H, 0, ch.keys, ch.vals, cap, ring[cur].H, 0, ring[cur].keys,
                                                 cap, P, c, c + 3, lgcur);
            if (join)
                k_spw_join<W><<<gc, 256, 0, st>>>(ch.keys, ch.vals, cap, cap, jH, (int)f[WK_JLG], jk,
                                                  (uint64_t)f[WK_JSTRIDE], T, res + i, c + 1, 0);
            int now = out;
            const unsigned long long *nnow = c;
            if (f[WK_TRUNC] >= 0) {
                // the cap drops at this cut: the whole table before the drop is joined too
                if (join)
                    k_spw_join<W><<<gc, 256, 0, st>>>(ring[out].keys, ring[out].vals, cap, cap, jH, (int)f[WK_JLG],
                                                      jk, (uint64_t)f[WK_JSTRIDE], T, res + i, c, SPW_TAG);
                const int tr = (out + 1) % 3;
                k_spw_fill_dyn<W><<<gi, 256, 0, st>>>(c, cap, 1, c + 5, ring[tr].H, nullptr, nullptr, abort);
                k_spw_filter<W><<<gc, 256, 0, st>>>(ring[out].keys, ring[out].vals, cap, cap, (int)f[WK_TRUNC],
                                                    ring[tr].keys, ring[tr].vals, cap, ring[tr].H, 0, c + 4, c, c + 5);
                now = tr;
                nnow = c + 4;
            }
            if (join) {
                pend = i;
                pend_out = out;
            }
            // keep mode 2 (small tables, a cache of the caller's) is left to the one-block walk
            if (f[WK_KEEP] == 1) {
                unsigned long long *rec = cnt + 8ull * (nsteps + 1 + i);
                k_spw_keep_alloc<<<1, 32, 0, st>>>(nnow, cap, W, (int)f[WK_KEEP], rec, used, arena ? arena_bytes : 0);
                k_spw_keep_fill<<<gi, 256, 0, st>>>(arena, rec, W);
                k_spw_keep<W><<<gc, 256, 0, st>>>(ring[now].keys, ring[now].vals, cap, nnow, arena, rec);
            }
            cur = now;
        }
        if (pend >= 0)
            k_spw_capture<W><<<1, 32, 0, st>>>(res + pend, ch.keys, ch.vals, ring[pend_out].keys, ring[pend_out].vals,
                                               cap, resk + (size_t)pend * W, resv + pend);
        e = cuda_check(cudaGetLastError(), "wide walk");
        if (e || i >= nsteps) return e;
        // the table size before step i (and whether a flag voided the walk)
        int noff, lgoff;
        const unsigned long long *pc = cnt + spw_prev_off(steps, i, noff, lgoff);
        e = cuda_check(cudaMemcpyAsync(hb, pc, 64, cudaMemcpyDeviceToHost, st), "walk read");
        if (!e) e = cuda_check(cudaMemcpyAsync(hb + 8, abort, 8, cudaMemcpyDeviceToHost, st), "walk read");
        if (!e) e = cuda_check(cudaStreamSynchronize(st), "walk sync");
        if (e) return e;
        if (hb[8]) break;
        host_n = std::min<uint64_t>(hb[noff], cap);
    }
    return cuda_check(cudaGetLastError(), "wide walk");
}

}  // namespace tg

using namespace tg;

#define SPW_DISPATCH(W, CALL)                    \
    switch (W) {                                  \
        case 1: return CALL(1);                   \
        case 2: return CALL(2);                   \
        case 3: return CALL(3);                   \
        case 4: return CALL(4);                   \
        case 5: return CALL(5);                   \
        case 6: return CALL(6);                   \
        case 7: return CALL(7);                   \
        default: return CALL(8);                  \
    }

extern "C" {

int tg_spw_step(int W, const void *keys, const void *vals, uint64_t n, uint64_t stride, const void *Hold, int lg_old,
                void *ekeys, void *evals, uint64_t ecap, void *Hs, int lgs, void *nkeys, void *nvals, uint64_t ncap,
                void *Hn, int lgn, void *ckeys, void *cvals, uint64_t ccap, const uint64_t *upd,
                const uint64_t *sel_mask, const uint64_t *sel_bits, int cap, int keep_below, int w, int want_changed,
                int use_h, int K, int ncls, const uint64_t *masks, const int64_t *weights, int64_t extra,
                const uint64_t *tmask, void *counters, void *stream) {
    int e = spw_check_words(W);
    if (e) return e;
    if (ecap < 2 * n || lgs < 1 || lgs > 40 || lgn < 1 || lgn > 40 || !counters || !upd || !sel_mask || !sel_bits ||
        (n && (!keys || !vals)) || !ekeys || !evals || !Hs || !nkeys || !nvals || !Hn ||
        (want_changed && (!ckeys || !cvals)) || w < 1 || cap > 254)
        return set_error(TG_ERR_ARG, "bad wide step arguments");
    if ((1ull << lgs) < 2 * n || ecap > SPW_IDX) return set_error(TG_ERR_TOO_BIG, "staging index too small");
    WideStep P;
    memset(&P, 0, sizeof(P));
    for (int q = 0; q < W; q++) {
        P.upd[q] = upd[q];
        P.sel_mask[q] = sel_mask[q];
        P.sel_bits[q] = sel_bits[q];
    }
    P.cap = cap;
    P.keep_below = keep_below;
    P.w = w;
    P.want_changed = want_changed;
    WideBound B;
    e = spw_bound(B, W, use_h, K, ncls, masks, weights, extra, tmask);
    if (e) return e;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
#define SPW_STEP(WW)                                                                                                  \
    spw_step_w<WW>((const uint64_t *)keys, (const uint8_t *)vals, n, stride, Hold, lg_old, (uint64_t *)ekeys,         \
                   (uint8_t *)evals, ecap, Hs, lgs, (uint64_t *)nkeys, (uint8_t *)nvals, ncap, Hn, lgn,              \
                   (uint64_t *)ckeys, (uint8_t *)cvals, ccap, P, B, counters, st)
    SPW_DISPATCH(W, SPW_STEP)
#undef SPW_STEP
}

// the one-block walk of wide tables runs while 2 n <= limit (0: never); returns the previous limit
int64_t tg_spw_set_small_limit(int64_t limit) {
    const int64_t old = (int64_t)g_spw_small_limit;
    if (limit >= 0) g_spw_small_limit = (uint64_t)limit;
    return old;
}

int64_t tg_spw_walk_scratch_bytes(int W, uint64_t cap, int nsteps) {
    if (spw_check_words(W) || cap < 1 || nsteps < 0) return -1;
    return (int64_t)spw_walk_layout(W, cap, nsteps, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                    nullptr);
}

// Run nsteps column steps from the table (keys0, vals0, n0 states, key stride stride0) on the device
// with one host read at the end.  Returns nsteps when done: out int64 [nsteps][6] = states after
// the step (and the cut's truncation), changed states, kept table's arena offset (-1: not kept),
// its key stride, its index bits (the working index's when not kept), states before the
// truncation; res uint64 [nsteps][2 + W] = least join total (all ones: none), the forward value,
// the forward key words.  Returns 0 with need[0] (states a table must hold) or need[1] (arena
// bytes) set when the tables or the arena were too small: the caller runs the leg again.
int tg_spw_walk(int W, int nsteps, const int64_t *steps, const uint64_t *words, const uint64_t *masks,
                const int64_t *weights, int maxc, int K, const void *keys0, const void *vals0, uint64_t n0,
                uint64_t stride0, void *scratch, uint64_t cap, void *arena, uint64_t arena_bytes, int64_t *out,
                uint64_t *res, int64_t *need, void *stream) {
    int e = spw_check_words(W);
    if (e) return e;
    if (nsteps < 0 || (nsteps && (!steps || !words || !out || !res)) || !scratch || !need || cap < 1 ||
        (n0 && (!keys0 || !vals0 || stride0 < n0)) || maxc < 1 || 2 * cap >= SPW_TAG)
        return set_error(TG_ERR_ARG, "bad wide walk arguments");
    need[0] = need[1] = 0;
    if (n0 > cap) {
        need[0] = (int64_t)n0;
        return 0;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint8_t *base = static_cast<uint8_t *>(scratch);
    unsigned long long *cnt, *resd;
    uint64_t *resk;
    uint8_t *resv;
    spw_walk_layout(W, cap, nsteps, base, nullptr, nullptr, nullptr, &cnt, &resd, &resk, &resv);
    const size_t bytes = (size_t)((resv + nsteps + 1) - reinterpret_cast<uint8_t *>(cnt));
    // pinned host buffer: the walk's reads of its state, then all its counters and results
    static thread_local uint8_t *hb = nullptr;
    static thread_local size_t hb_bytes = 0;
    const size_t want = std::max<size_t>(bytes, 128);
    if (hb_bytes < want) {
        if (hb) cudaFreeHost(hb);
        hb = nullptr;
        hb_bytes = 0;
        if (cudaMallocHost(&hb, want) != cudaSuccess) {
            cudaGetLastError();
            return set_error(TG_ERR_NOMEM, "pinned walk buffer");
        }
        hb_bytes = want;
    }
    unsigned long long *hsmall = reinterpret_cast<unsigned long long *>(hb);
#define SPW_WALK(WW)                                                                                                  \
    spw_walk_w<WW>(nsteps, steps, words, masks, weights, maxc, K, (const uint64_t *)keys0, (const uint8_t *)vals0, n0, \
                   stride0, base, cap, (uint8_t *)arena, arena_bytes, hsmall, st)
    auto run = [&]() -> int { SPW_DISPATCH(W, SPW_WALK) };
#undef SPW_WALK
    e = run();
    if (e) return e;
    e = cuda_check(cudaMemcpyAsync(hb, cnt, bytes, cudaMemcpyDeviceToHost, st), "walk read");
    if (!e) e = cuda_check(cudaStreamSynchronize(st), "walk sync");
    if (e) return e;
    const unsigned long long *hc = reinterpret_cast<const unsigned long long *>(hb);
    const uint8_t *hr = hb + (reinterpret_cast<uint8_t *>(resd) - reinterpret_cast<uint8_t *>(cnt));
    const unsigned long long *hres = reinterpret_cast<const unsigned long long *>(hr);
    const uint64_t *hk = reinterpret_cast<const uint64_t *>(hb + (reinterpret_cast<uint8_t *>(resk) -
                                                                  reinterpret_cast<uint8_t *>(cnt)));
    const uint8_t *hv = hb + (resv - reinterpret_cast<uint8_t *>(cnt));
    uint64_t most = hc[0];
    bool small = (hc[2] & 7ull) != 0, room = false;
    for (int i = 0; i < nsteps; i++) {
        const unsigned long long *c = hc + 8ull * (i + 1), *rec = hc + 8ull * (nsteps + 1 + i);
        most = std::max<uint64_t>(most, std::max<uint64_t>(c[0], std::max<uint64_t>(c[1], c[4])));
        small = small || ((c[2] | c[6] | rec[2]) & 7ull);
        room = room || (rec[2] & 8ull);
    }
    if (small) {
        need[0] = (int64_t)std::max<uint64_t>(2 * cap, most + 1);
        return 0;
    }
    if (room) {
        need[1] = (int64_t)hc[8ull * (2 * (uint64_t)nsteps + 1)];
        return 0;
    }
    for (int i = 0; i < nsteps; i++) {
        const int64_t *f = steps + (size_t)SPW_WALK_FIELDS * i;
        const unsigned long long *c = hc + 8ull * (i + 1), *rec = hc + 8ull * (nsteps + 1 + i);
        // kept: placed in the arena (the separate-launch path leaves keep mode 2 to the one-block walk)
        const bool tr = f[WK_TRUNC] >= 0, kept = f[WK_KEEP] && !(rec[2] & 16ull) && rec[4] != 0;
        int64_t *o = out + 6 * (size_t)i;
        o[0] = (int64_t)(tr ? c[4] : c[0]);
        o[1] = (int64_t)c[1];
        o[2] = kept ? (int64_t)rec[1] : -1;
        o[3] = kept ? (int64_t)rec[4] : (int64_t)cap;
        o[4] = kept ? (int64_t)rec[3] : (int64_t)(tr ? c[5] : c[3]);
        o[5] = (int64_t)c[0];
        uint64_t *r = res + (size_t)(2 + W) * i;
        r[0] = hres[i] == SPW_EMPTY ? SPW_EMPTY : hres[i] >> 40;
        r[1] = hv[i];
        for (int q = 0; q < W; q++) r[2 + q] = hk[(size_t)i * W + q];
    }
    return nsteps;
}

int tg_spw_filter(int W, const void *keys, const void *vals, uint64_t n, uint64_t stride, int below, void *nkeys,
                  void *nvals, uint64_t ncap, void *Hn, int lgn, void *counters, void *stream) {
    int e = spw_check_words(W);
    if (e) return e;
    if ((n && (!keys || !vals)) || !nkeys || !nvals || !Hn || lgn < 1 || lgn > 40 || !counters || ncap < 1)
        return set_error(TG_ERR_ARG, "bad wide filter arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned long long *C = (unsigned long long *)counters;
    e = cuda_check(cudaMemsetAsync(C, 0, 4 * sizeof(unsigned long long), st), "counters");
    if (e) return e;
    k_spw_fill<<<spw_grid(1ull << lgn), 256, 0, st>>>((unsigned long long *)Hn, 1ull << lgn);
    if (n) {
#define SPW_FILTER(WW)                                                                                                \
    (k_spw_filter<WW><<<spw_grid(n), 256, 0, st>>>((const uint64_t *)keys, (const uint8_t *)vals, n, stride, below,  \
                                                    (uint64_t *)nkeys, (uint8_t *)nvals, ncap,                        \
                                                    (unsigned long long *)Hn, lgn, C),                                \
     cuda_check(cudaGetLastError(), "wide filter"))
        SPW_DISPATCH(W, SPW_FILTER)
#undef SPW_FILTER
    }
    return cuda_check(cudaGetLastError(), "wide filter");
}

int tg_spw_join(int W, const void *fkeys, const void *fvals, uint64_t nf, uint64_t fstride, const void *Hb, int lgb,
                const void *bkeys, uint64_t bstride, const uint64_t *tmask, void *result, void *stream) {
    int e = spw_check_words(W);
    if (e) return e;
    if (!result || !Hb || !bkeys || (nf && (!fkeys || !fvals)) || !tmask || lgb < 1 || lgb > 40)
        return set_error(TG_ERR_ARG, "bad wide join arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    e = cuda_check(cudaMemsetAsync(result, 0xFF, sizeof(unsigned long long), st), "join result");
    if (e || !nf) return e;
    WideBound T;
    memset(&T, 0, sizeof(T));
    for (int q = 0; q < W; q++) T.tmask[q] = tmask[q];
#define SPW_JOIN(WW)                                                                                                  \
    (k_spw_join<WW><<<spw_grid(nf), 256, 0, st>>>((const uint64_t *)fkeys, (const uint8_t *)fvals, nf, fstride,      \
                                                   (const unsigned long long *)Hb, lgb, (const uint64_t *)bkeys,      \
                                                   bstride, T, (unsigned long long *)result),                         \
     cuda_check(cudaGetLastError(), "wide join"))
    SPW_DISPATCH(W, SPW_JOIN)
#undef SPW_JOIN
}

int tg_spw_lookup(int W, const void *H, int lg, const void *keys, uint64_t stride, const void *q, uint64_t m,
                  void *out, void *stream) {
    int e = spw_check_words(W);
    if (e) return e;
    if (!H || !keys || (m && (!q || !out)) || lg < 1 || lg > 40) return set_error(TG_ERR_ARG, "bad wide lookup");
    if (!m) return TG_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
#define SPW_LOOK(WW)                                                                                                  \
    (k_spw_lookup<WW><<<spw_grid(m), 256, 0, st>>>((const unsigned long long *)H, lg, (const uint64_t *)keys, stride,\
                                                    (const uint64_t *)q, m, (uint8_t *)out),                          \
     cuda_check(cudaGetLastError(), "wide lookup"))
    SPW_DISPATCH(W, SPW_LOOK)
#undef SPW_LOOK
}

}  // extern "C"
