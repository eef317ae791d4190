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
    int sel_any;                // sel_mask != 0
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

template <int W>
__device__ __forceinline__ bool spw_equal(const uint64_t *keys, uint64_t stride, uint64_t i, const uint64_t (&k)[W]) {
    bool eq = true;
#pragma unroll
    for (int w = 0; w < W; w++) eq = eq && keys[(uint64_t)w * stride + i] == k[w];
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
        const unsigned long long cur = H[s];
        if (cur == SPW_EMPTY) return 255u;
        if (spw_equal<W>(keys, stride, cur & SPW_IDX, k)) return (uint32_t)(cur >> 56);
        s = (s + 1) & mask;
    }
    return 255u;
}

// staging: write the key, then insert value << 56 | e keeping the least word per key
template <int W>
__device__ __forceinline__ void spw_emit(uint64_t *ek, uint64_t estride, uint8_t *ev, unsigned long long *H, int lg,
                                         uint64_t e, const uint64_t (&k)[W], uint32_t v, unsigned long long *err) {
#pragma unroll
    for (int w = 0; w < W; w++) __stcg(ek + (uint64_t)w * estride + e, k[w]);
    ev[e] = (uint8_t)v;
    __threadfence();
    const unsigned long long word = ((unsigned long long)v << 56) | e;
    const uint32_t mask = (1u << lg) - 1u;
    uint32_t s = spw_slot<W>(k, lg);
    for (uint32_t probe = 0; probe <= mask; probe++) {
        unsigned long long cur = atomicCAS(H + s, SPW_EMPTY, word);
        if (cur == SPW_EMPTY) return;
        __threadfence();
        if (spw_equal_cg<W>(ek, estride, cur & SPW_IDX, k)) {
            atomicMin(H + s, word);
            return;
        }
        s = (s + 1) & mask;
    }
    atomicOr(err, 1ull);
}

__global__ void k_spw_fill(unsigned long long *H, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        H[i] = SPW_EMPTY;
}

template <int W>
__global__ void k_spw_emit(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ vals, uint64_t n,
                           uint64_t stride, uint64_t *ek, uint8_t *ev, uint64_t estride, unsigned long long *H, int lg,
                           const WideStep P, const WideBound B, unsigned long long *counters) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
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
            if ((int)v <= P.cap && spw_keep<W>(B, c, v)) spw_emit<W>(ek, estride, ev, H, lg, 2 * i, c, v, counters + 2);
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
            if (any && cpass && spw_keep<W>(B, c, cv)) spw_emit<W>(ek, estride, ev, H, lg, 2 * i + 1, c, cv, counters + 2);
        }
    }
}

// new table (keys, vals, index lg2) from the staging index; changed states from candidate slots
template <int W>
__global__ void k_spw_compact(const unsigned long long *__restrict__ H, uint64_t hcap, const uint64_t *__restrict__ ek,
                              uint64_t estride, uint64_t *nk, uint8_t *nv, uint64_t ncap, unsigned long long *H2,
                              int lg2, uint64_t *ck, uint8_t *cv, uint64_t ccap, const unsigned long long *Hold,
                              int lg_old, const uint64_t *okeys, uint64_t ostride, const WideStep P,
                              unsigned long long *counters) {
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < hcap; s += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long cur = H[s];
        if (cur == SPW_EMPTY) continue;
        const uint64_t e = cur & SPW_IDX;
        const uint32_t v = (uint32_t)(cur >> 56);
        uint64_t k[W];
        spw_load<W>(ek, estride, e, k);
        if (P.want_changed && (e & 1ull)) {
            // a candidate won: changed unless the old table had this key (closing bits restored)
            // with a value <= v
            uint64_t o[W];
#pragma unroll
            for (int w = 0; w < W; w++) o[w] = k[w] | P.sel_bits[w];
            if (v < spw_lookup<W>(Hold, lg_old, okeys, ostride, o)) {
                const unsigned long long j = atomicAdd(counters + 1, 1ull);
                if (j < ccap) {
#pragma unroll
                    for (int w = 0; w < W; w++) ck[(uint64_t)w * ccap + j] = k[w];
                    cv[j] = (uint8_t)v;
                } else {
                    atomicOr(counters + 2, 2ull);
                }
            }
        }
        if (P.keep_below >= 0 && (int)v >= P.keep_below) continue;
        const unsigned long long j = atomicAdd(counters, 1ull);
        if (j >= ncap) { atomicOr(counters + 2, 4ull); continue; }
#pragma unroll
        for (int w = 0; w < W; w++) nk[(uint64_t)w * ncap + j] = k[w];
        nv[j] = (uint8_t)v;
        // the keys are distinct: claim the first empty slot
        const uint32_t mask = (1u << lg2) - 1u;
        uint32_t t = spw_slot<W>(k, lg2);
        uint32_t probe = 0;
        for (; probe <= mask; probe++) {
            if (atomicCAS(H2 + t, SPW_EMPTY, ((unsigned long long)v << 56) | j) == SPW_EMPTY) break;
            t = (t + 1) & mask;
        }
        if (probe > mask) atomicOr(counters + 2, 1ull);
    }
}

// a table's states with value < below, with their own index
template <int W>
__global__ void k_spw_filter(const uint64_t *__restrict__ keys, const uint8_t *__restrict__ vals, uint64_t n,
                             uint64_t stride, int below, uint64_t *nk, uint8_t *nv, uint64_t ncap,
                             unsigned long long *H2, int lg2, unsigned long long *counters) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = vals[i];
        if (below >= 0 && (int)v >= below) continue;
        uint64_t k[W];
        spw_load<W>(keys, stride, i, k);
        const unsigned long long j = atomicAdd(counters, 1ull);
        if (j >= ncap) { atomicOr(counters + 2, 4ull); continue; }
#pragma unroll
        for (int w = 0; w < W; w++) nk[(uint64_t)w * ncap + j] = k[w];
        nv[j] = (uint8_t)v;
        const uint32_t mask = (1u << lg2) - 1u;
        uint32_t t = spw_slot<W>(k, lg2);
        uint32_t probe = 0;
        for (; probe <= mask; probe++) {
            if (atomicCAS(H2 + t, SPW_EMPTY, ((unsigned long long)v << 56) | j) == SPW_EMPTY) break;
            t = (t + 1) & mask;
        }
        if (probe > mask) atomicOr(counters + 2, 1ull);
    }
}

// least f.value + b.value over changed f and backward b with key(b) = key(f) ^ tmask:
// result = min(total << 40 | f)
template <int W>
__global__ void k_spw_join(const uint64_t *__restrict__ fk, const uint8_t *__restrict__ fv, uint64_t nf,
                           uint64_t fstride, const unsigned long long *__restrict__ Hb, int lgb,
                           const uint64_t *__restrict__ bk, uint64_t bstride, const WideBound T,
                           unsigned long long *result) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nf; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t q[W];
        spw_load<W>(fk, fstride, i, q);
#pragma unroll
        for (int w = 0; w < W; w++) q[w] ^= T.tmask[w];
        const uint32_t bv = spw_lookup<W>(Hb, lgb, bk, bstride, q);
        if (bv == 255u) continue;
        atomicMin(result, ((unsigned long long)(fv[i] + bv) << 40) | i);
    }
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
