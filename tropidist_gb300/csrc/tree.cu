// Exact min-plus tree DP on the GPU (cdist/tree_dp.c:13-43, cdist/tree_dp.py:409-501).
//
// A binary tree over the columns has one table per node, indexed by the node's interface state;
// a join enumerates the 2^J compatible (left, right) state pairs of a node, J = P + F: generators
// 0..P-1 lift the parent's unit vectors, generators P..J-1 span the kernel of child addition.
// Pair x in [0, 2^J) has left state XOR(lmap[i] : bit i of x), right state XOR(rmap[i]) and parent
// x & (2^P - 1); the parent entry is the least left + right over its pairs (entries < INF =
// ncols + 1; a finite sum never reaches INF, since the two subtrees' columns are disjoint).
//
// Device tables are uint32 in one arena.  The host indexes both children of a join in bases that
// start with their common part, so the kernel generators are unit pairs and a parent's pairs read
// aligned 2^F-entry blocks of each child.  A tree plan (host-built) lists the leaves and the joins
// grouped by height, all joins of one height in one launch of
//   - k_tree_small: one block runs a whole run of consecutive small heights (a few thousand
//     pairs each, e.g. the long spine of a comb tree) with a block barrier between heights;
//   - k_tree_gemm: a join whose parents cover every pair of child blocks, as a tiled min-plus
//     matrix product of XOR-permuted child rows through shared memory;
//   - k_tree_fill + k_tree_join for the other joins: lane groups of 2^F lanes per parent (F <= 4),
//     a warp per parent (F >= 5), or per-thread Gray walks of 2^R pairs of one parent; when a
//     parent's pairs span threads they are reduced across the warp and committed with atomicMin
//     into a table pre-filled with INF.
// The reference's per-call entry points (tree_join_u8/u16/u32/u64 over a pair range, tree_move)
// are provided on device pointers with the reference's argument meaning.
#include "tg_common.cuh"
#include "tg_capi.h"

#include <algorithm>
#include <cstring>
#include <vector>

namespace tg {

#define TR_MAXJ 62
#define TR_SMALL_PAIRS (1ll << 15)     // default: heights of at most this many pairs run in k_tree_small
#define TR_BS 256

struct TJoin {                 // one join of a tree plan (device)
    int64_t lo, ro, po;        // arena offsets (entries) of the left, right and parent tables
    int64_t block0;            // first block of this join in its launch (k_tree_join)
    int32_t P, F, R, mapoff;   // parent rank, kernel generators, pair bits per thread (warp), maps index
    int32_t W, pad;            // W = 1: the lanes of a warp take kernel generators 0..4 of one parent;
                               // W = 2 (F <= 4): 2^F lanes per parent, 2^R parents per lane
};

struct TFill { int64_t po, size, block0; };

// ---------------------------------------------------------------- leaves
// leaves: rows (offset, size, column, nonzero); the table of a leaf is [bit] or [bit, bit ^ 1] for
// the target representative's bit of that column, [0] for a zero column (cdist/tree_dp.py:465-471)
__global__ void k_tree_leaves(const int64_t *leaves, int64_t n, const uint64_t *target, uint32_t *arena) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t off = leaves[4 * i], size = leaves[4 * i + 1], col = leaves[4 * i + 2], nz = leaves[4 * i + 3];
    const uint32_t bit = (uint32_t)((target[col >> 6] >> (col & 63)) & 1ull);
    arena[off] = nz ? bit : 0u;
    if (size == 2) arena[off + 1] = bit ^ 1u;
}

// ---------------------------------------------------------------- one small join by a group of lanes
// pairs x = g, g + stride, ... of one join; state from the set bits of x (J small here)
__device__ __forceinline__ void small_pairs(const TJoin &d, const uint32_t *maps, uint32_t *arena, uint32_t inf,
                                            int g, int stride) {
    const int J = d.P + d.F;
    const uint32_t pmask = (1u << d.P) - 1u;
    const uint32_t *lm = maps + 2 * d.mapoff;
    const uint64_t npairs = 1ull << J;
    for (uint64_t x = (uint64_t)g; x < npairs; x += (uint64_t)stride) {
        uint32_t li = 0, ri = 0;
        for (uint64_t y = x; y; y &= y - 1) {
            const int b = __ffsll((long long)y) - 1;
            li ^= lm[2 * b];
            ri ^= lm[2 * b + 1];
        }
        const uint32_t c = arena[d.lo + li] + arena[d.ro + ri];
        if (d.F == 0) arena[d.po + (x & pmask)] = min(c, inf);
        else if (c < inf) atomicMin(arena + d.po + (x & pmask), c);
    }
}

// heights [h0, h1) of the plan in one block: lvl[h] .. lvl[h + 1] are the joins of height h
__global__ void __launch_bounds__(1024) k_tree_small(const TJoin *joins, const int64_t *lvl, int h0, int h1,
                                                     const uint32_t *maps, uint32_t *arena, uint32_t inf) {
    const int t = threadIdx.x, nt = blockDim.x, warp = t >> 5, lane = t & 31, nw = nt >> 5;
    for (int h = h0; h < h1; h++) {
        const int64_t j0 = lvl[h], j1 = lvl[h + 1];
        // parents whose pairs are spread over lanes start at INF
        for (int64_t j = j0; j < j1; j++) {
            const TJoin d = joins[j];
            if (d.F == 0) continue;
            for (int64_t e = t; e < (1ll << d.P); e += nt) arena[d.po + e] = inf;
        }
        __syncthreads();
        if (j1 - j0 >= nw) {
            for (int64_t j = j0 + warp; j < j1; j += nw) small_pairs(joins[j], maps, arena, inf, lane, 32);
        } else {
            for (int64_t j = j0; j < j1; j++) small_pairs(joins[j], maps, arena, inf, t, nt);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- large heights
__global__ void k_tree_fill(const TFill *fills, int nf, uint32_t *arena, uint32_t inf) {
    __shared__ int sf;
    if (threadIdx.x == 0) {
        int lo = 0, hi = nf - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (fills[mid].block0 <= (int64_t)blockIdx.x) lo = mid; else hi = mid - 1;
        }
        sf = lo;
    }
    __syncthreads();
    const TFill f = fills[sf];
    const int64_t base = ((int64_t)blockIdx.x - f.block0) * (int64_t)(TR_BS * 8);
    for (int k = 0; k < 8; k++) {
        const int64_t e = base + (int64_t)k * TR_BS + threadIdx.x;
        if (e < f.size) arena[f.po + e] = inf;
    }
}

template <int RI>
__device__ __forceinline__ uint32_t gray_walk(uint32_t m, uint32_t li, uint32_t ri, const uint32_t *gl,
                                              const uint32_t *L, const uint32_t *Rt) {
    // pairs base ^ gray(k), k = 0 .. 2^RI - 1; generator of step k is ctz(k)
    uint32_t a[RI > 0 ? RI : 1], b[RI > 0 ? RI : 1];
#pragma unroll
    for (int i = 0; i < RI; i++) { a[i] = gl[2 * i]; b[i] = gl[2 * i + 1]; }
    // batches of up to 8 pairs: all 16 gathers of a batch are issued before any is used, so a warp
    // keeps many L2 requests in flight (the kernel is bound by gather latency, not bandwidth)
    constexpr int NB = (1 << RI) < 8 ? (1 << RI) : 8;
#pragma unroll
    for (int k0 = 0; k0 < (1 << RI); k0 += NB) {
        uint32_t x[NB], y[NB];
#pragma unroll
        for (int k = k0; k < k0 + NB; k++) {
            if (k) {
                const int bit = __ffs(k) - 1;        // a constant once unrolled
                li ^= a[bit];
                ri ^= b[bit];
            }
            x[k - k0] = __ldg(L + li);
            y[k - k0] = __ldg(Rt + ri);
        }
#pragma unroll
        for (int k = 0; k < NB; k++) m = min(m, x[k] + y[k]);
    }
    return m;
}

// The parents (pc << PW) | g, g < 2^PW, of one lane group (2^F lanes, lane f = pair f), pc = u >> F:
// parent k of the walk (Gray order) toggles parent generator ctz(k); all lanes of the warp run the
// same steps (the shuffles need them), lanes past nthr only compute dummies.
template <int PW>
__device__ __forceinline__ void group_walk(const TJoin &d, uint64_t u, uint64_t nthr, const uint32_t *sg,
                                           const uint32_t *L, const uint32_t *Rt, uint32_t *arena, uint32_t inf) {
    const int F = d.F;
    const uint32_t f = threadIdx.x & ((1u << F) - 1u);
    const bool active = u < nthr;
    const uint64_t pc = u >> F;
    uint32_t bl = 0, br = 0;
    if (active)
        for (uint64_t y = (pc << PW) | ((uint64_t)f << d.P); y; y &= y - 1) {
            const int b = __ffsll((long long)y) - 1;
            bl ^= sg[2 * b];
            br ^= sg[2 * b + 1];
        }
    uint32_t gl[PW > 0 ? PW : 1], gr[PW > 0 ? PW : 1];
#pragma unroll
    for (int b = 0; b < PW; b++) { gl[b] = sg[2 * b]; gr[b] = sg[2 * b + 1]; }
    uint32_t res[1 << PW];
#pragma unroll
    for (int k = 0; k < (1 << PW); k++) {
        if (k) {
            const int b = __ffs(k) - 1;                // a constant once unrolled
            bl ^= gl[b];
            br ^= gr[b];
        }
        uint32_t v = active ? __ldg(L + bl) + __ldg(Rt + br) : inf;
        for (int off = 1; off < (1 << F); off <<= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, off));
        res[k ^ (k >> 1)] = min(v, inf);
    }
    if (active && f == 0) {
        uint32_t *out = arena + d.po + (pc << PW);
#pragma unroll
        for (int k = 0; k < (1 << PW); k++) out[k] = res[k];
    }
}

__global__ void __launch_bounds__(TR_BS, 3) k_tree_join(const TJoin *joins, int nj, const uint32_t *maps,
                                                     uint32_t *arena, uint32_t inf) {
    __shared__ uint32_t sg[2 * TR_MAXJ];
    __shared__ int sj;
    if (threadIdx.x == 0) {
        int lo = 0, hi = nj - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (joins[mid].block0 <= (int64_t)blockIdx.x) lo = mid; else hi = mid - 1;
        }
        sj = lo;
    }
    __syncthreads();
    const TJoin d = joins[sj];
    const int J = d.P + d.F;
    for (int i = threadIdx.x; i < 2 * J; i += TR_BS) sg[i] = maps[2 * d.mapoff + i];
    __syncthreads();
    if (d.W == 1) {
        // warp mode (F >= 5): a warp takes 2^R pairs of one parent, lane l the pairs whose kernel
        // generators 0..4 are the bits of l; with unit kernel generators the lanes read consecutive
        // entries at every step
        const int RW = d.R - 5, RI = min(RW, 6), RO = RW - RI;
        const uint64_t nthr = 1ull << (J - d.R + 5);
        const uint64_t u = ((uint64_t)blockIdx.x - (uint64_t)d.block0) * TR_BS + threadIdx.x;
        const uint32_t lane = threadIdx.x & 31u;
        const uint64_t w = u >> 5, p = w & ((1ull << d.P) - 1ull);
        uint32_t m = inf;
        if (u < nthr) {
            const uint64_t x0 = p | ((uint64_t)lane << d.P) | ((w >> d.P) << (d.P + d.R));
            uint32_t bl = 0, br = 0;
            for (uint64_t y = x0; y; y &= y - 1) {
                const int b = __ffsll((long long)y) - 1;
                bl ^= sg[2 * b];
                br ^= sg[2 * b + 1];
            }
            const uint32_t *L = arena + d.lo, *Rt = arena + d.ro;
            const uint32_t *gi = sg + 2 * (d.P + 5);
            for (uint64_t q = 0; q < (1ull << RO); q++) {
                if (q) {
                    const int b = d.P + 5 + RI + __ffsll((long long)q) - 1;
                    bl ^= sg[2 * b];
                    br ^= sg[2 * b + 1];
                }
                switch (RI) {
                    case 0: m = gray_walk<0>(m, bl, br, gi, L, Rt); break;
                    case 1: m = gray_walk<1>(m, bl, br, gi, L, Rt); break;
                    case 2: m = gray_walk<2>(m, bl, br, gi, L, Rt); break;
                    case 3: m = gray_walk<3>(m, bl, br, gi, L, Rt); break;
                    case 4: m = gray_walk<4>(m, bl, br, gi, L, Rt); break;
                    case 5: m = gray_walk<5>(m, bl, br, gi, L, Rt); break;
                    default: m = gray_walk<6>(m, bl, br, gi, L, Rt); break;
                }
            }
        }
        for (int off = 16; off > 0; off >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, off));
        if (lane == 0 && u < nthr) {
            if (d.F == d.R) arena[d.po + p] = min(m, inf);
            else if (m < inf) atomicMin(arena + d.po + p, m);
        }
        return;
    }
    if (d.W == 2) {
        // small kernel (F <= 4): a group of 2^F lanes takes one parent, lane f its pair f, so the
        // group reads one aligned 2^F-entry block of each child (one sector); every thread walks 2^PW
        // consecutive parents in Gray order (one parent generator toggled per parent, the XOR of the
        // first parent's generators paid once), the group minimum comes from F shuffles, and the
        // group's first lane writes its 2^PW parents as one vector
        const uint64_t u = ((uint64_t)blockIdx.x - (uint64_t)d.block0) * TR_BS + threadIdx.x;
        const uint64_t nthr = 1ull << (d.P - d.R + d.F);
        const uint32_t *L = arena + d.lo, *Rt = arena + d.ro;
        switch (d.R) {
            case 0: group_walk<0>(d, u, nthr, sg, L, Rt, arena, inf); break;
            case 1: group_walk<1>(d, u, nthr, sg, L, Rt, arena, inf); break;
            case 2: group_walk<2>(d, u, nthr, sg, L, Rt, arena, inf); break;
            case 3: group_walk<3>(d, u, nthr, sg, L, Rt, arena, inf); break;
            default: group_walk<4>(d, u, nthr, sg, L, Rt, arena, inf); break;
        }
        return;
    }
    const int R = d.R, RI = min(R, 6), RO = R - RI;
    const uint64_t nthr = 1ull << (J - R);
    const uint64_t u = ((uint64_t)blockIdx.x - (uint64_t)d.block0) * TR_BS + threadIdx.x;
    const uint64_t pm = (1ull << d.P) - 1ull;
    uint32_t m = inf;
    const uint64_t p = u & pm;
    if (u < nthr) {
        // thread u: parent p = low P bits, pair chunk fc = the rest; first pair x0 = p | fc << (P + R)
        const uint64_t x0 = p | ((u >> d.P) << (d.P + R));
        uint32_t bl = 0, br = 0;
        for (uint64_t y = x0; y; y &= y - 1) {
            const int b = __ffsll((long long)y) - 1;
            bl ^= sg[2 * b];
            br ^= sg[2 * b + 1];
        }
        // start each lane at its own offset inside the inner walk (the same pairs in another order),
        // so the lanes of a warp do not all touch the same offset of their blocks at once
        for (uint32_t c = threadIdx.x & ((1u << RI) - 1u), b = 0; c; c >>= 1, b++)
            if (c & 1u) {
                bl ^= sg[2 * (d.P + b)];
                br ^= sg[2 * (d.P + b) + 1];
            }
        const uint32_t *L = arena + d.lo, *Rt = arena + d.ro;
        const uint32_t *gi = sg + 2 * d.P;             // the RI inner generators
        for (uint64_t q = 0; q < (1ull << RO); q++) {
            if (q) {                                   // outer Gray step over generators P + RI ..
                const int b = d.P + RI + __ffsll((long long)q) - 1;
                bl ^= sg[2 * b];
                br ^= sg[2 * b + 1];
            }
            switch (RI) {
                case 0: m = gray_walk<0>(m, bl, br, gi, L, Rt); break;
                case 1: m = gray_walk<1>(m, bl, br, gi, L, Rt); break;
                case 2: m = gray_walk<2>(m, bl, br, gi, L, Rt); break;
                case 3: m = gray_walk<3>(m, bl, br, gi, L, Rt); break;
                case 4: m = gray_walk<4>(m, bl, br, gi, L, Rt); break;
                case 5: m = gray_walk<5>(m, bl, br, gi, L, Rt); break;
                default: m = gray_walk<6>(m, bl, br, gi, L, Rt); break;
            }
        }
    }
    if (d.F <= R) {                                    // the thread owns its parent entry
        if (u < nthr) arena[d.po + p] = min(m, inf);
        return;
    }
    if (d.P < 5) {                                     // lanes u ^ (k << P) share the parent
        for (int off = 1 << d.P; off < 32; off <<= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, off));
        if ((threadIdx.x & 31) >= (1 << d.P)) return;
    }
    if (u < nthr && m < inf) atomicMin(arena + d.po + p, m);
}

// ---------------------------------------------------------------- joins as min-plus block products
// When the kernel generators are the unit pairs (e_k, e_k) and every left block meets every right
// block, parent p = PA a ^ PB b ^ PT t reads left row a and right row b (2^F entries each) with
// XOR offsets DL a and DR b ^ DT t, and its value is min over f of L'[a][f] + R'[b][f]: a min-plus
// matrix product, tiled through shared memory (a 64 x 64 tile of parents per block, 16 per thread,
// K in chunks of 32 staged with the offsets applied), every parent written once.
#define TG_T 64
#define TG_KC 32
#define TG_LD (TG_T + 4)

struct TGemm {
    int64_t lo, ro, po;                // arena offsets of the left, right and parent tables
    int32_t F, mb, nb, kb;             // row length 2^F, 2^mb left rows, 2^nb right rows, 2^kb products
    int32_t mapoff, pad;               // DL[mb] DR[nb] DT[kb] PA[mb] PB[nb] PT[kb] at gmaps[mapoff]
};

__device__ __forceinline__ uint32_t xor_bits(const uint32_t *v, int n, uint32_t x) {
    uint32_t o = 0;
    for (int i = 0; i < n; i++)
        if ((x >> i) & 1u) o ^= v[i];
    return o;
}

// PACK (INF < 2^15): right entries staged as 16-bit pairs, two parents per __viaddmin_u16x2 with
// the left entry duplicated into both halves by an IMAD (FMA pipe); otherwise one per __viaddmin_u32.
// KC = min(32, 2^F) entries of every row per chunk; the staging is double-buffered: chunk k + 1 is
// loaded while chunk k is reduced.
template <int N>
__device__ __forceinline__ void load_entries(const uint32_t *p, uint32_t (&v)[N]) {
    if constexpr (N == 8) {
        const uint4 a = __ldg(reinterpret_cast<const uint4 *>(p)), b = __ldg(reinterpret_cast<const uint4 *>(p) + 1);
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    } else if constexpr (N == 4) {
        const uint4 a = __ldg(reinterpret_cast<const uint4 *>(p));
        v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
    } else if constexpr (N == 2) {
        const uint2 a = __ldg(reinterpret_cast<const uint2 *>(p));
        v[0] = a.x; v[1] = a.y;
    } else {
        v[0] = __ldg(p);
    }
}

template <bool PACK, int KC>
__global__ void __launch_bounds__(256) k_tree_gemm(const __grid_constant__ TGemm G, const uint32_t *gmaps,
                                                   uint32_t *arena, uint32_t inf) {
    constexpr int NE = KC / 4;          // entries of a row staged by one thread per chunk
    __shared__ __align__(16) uint32_t As[2][KC][TG_LD];
    __shared__ __align__(16) uint32_t Bs[2][KC][PACK ? TG_LD / 2 : TG_LD];
    __shared__ uint32_t dl[TG_T], dr[TG_T];
    const uint32_t *DL = gmaps + G.mapoff, *DR = DL + G.mb, *DT = DR + G.nb;
    const uint32_t *PA = DT + G.kb, *PB = PA + G.mb, *PT = PB + G.nb;
    const uint32_t a0 = blockIdx.y * TG_T, b0 = blockIdx.x * TG_T, t = blockIdx.z;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    if (tid < TG_T) dl[tid] = xor_bits(DL, G.mb, a0 + tid);
    else if (tid < 2 * TG_T) dr[tid - TG_T] = xor_bits(DR, G.nb, b0 + tid - TG_T) ^ xor_bits(DT, G.kb, t);
    __syncthreads();
    // staging: thread -> row r = tid / 4 of the tile, entries NE q .. NE q + NE - 1 of the chunk's
    // aligned group; entry k0 + j of row a is L[a][(k0 + j) ^ dl] = group (k0 ^ (dl & ~(KC - 1))),
    // element j ^ (dl & (KC - 1))
    const int r = tid >> 2, q = tid & 3;
    const uint32_t dla = dl[r], drb = dr[r];
    const uint32_t *Lrow = arena + G.lo + ((uint64_t)(a0 + r) << G.F);
    const uint32_t *Rrow = arena + G.ro + ((uint64_t)(b0 + r) << G.F);
    const uint32_t nk = 1u << G.F, km = (uint32_t)KC - 1u;
    uint32_t xa[NE], yb[NE];
    auto fetch = [&](uint32_t k0) {
        load_entries<NE>(Lrow + ((k0 ^ (dla & ~km)) + NE * q), xa);
        load_entries<NE>(Rrow + ((k0 ^ (drb & ~km)) + NE * q), yb);
    };
    auto stage = [&](int buf) {
#pragma unroll
        for (int e = 0; e < NE; e++) {
            As[buf][(NE * q + e) ^ (dla & km)][r] = xa[e];
            if (PACK) reinterpret_cast<uint16_t *>(&Bs[buf][(NE * q + e) ^ (drb & km)][0])[r] = (uint16_t)yb[e];
            else Bs[buf][(NE * q + e) ^ (drb & km)][r] = yb[e];
        }
    };
    uint32_t acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = PACK ? (inf | (inf << 16)) : inf;
    fetch(0);
    stage(0);
    __syncthreads();
    int buf = 0;
    for (uint32_t k0 = 0; k0 < nk; k0 += KC) {
        const bool more = k0 + KC < nk;
        if (more) fetch(k0 + KC);
#pragma unroll 8
        for (int kk = 0; kk < KC; kk++) {
            const uint4 a = *reinterpret_cast<const uint4 *>(&As[buf][kk][4 * ty]);
            const uint32_t av[4] = {a.x, a.y, a.z, a.w};
            if (PACK) {
                const uint2 b = *reinterpret_cast<const uint2 *>(&Bs[buf][kk][2 * tx]);
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    const uint32_t ad = av[i] * 0x10001u;
                    acc[i][0] = __viaddmin_u16x2(ad, b.x, acc[i][0]);
                    acc[i][1] = __viaddmin_u16x2(ad, b.y, acc[i][1]);
                }
            } else {
                const uint4 b = *reinterpret_cast<const uint4 *>(&Bs[buf][kk][4 * tx]);
                const uint32_t bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) acc[i][j] = __viaddmin_u32(av[i], bv[j], acc[i][j]);
            }
        }
        if (more) stage(buf ^ 1);
        __syncthreads();
        buf ^= 1;
    }
    const uint32_t pt = xor_bits(PT, G.kb, t);
    uint32_t pb[4];
#pragma unroll
    for (int j = 0; j < 4; j++) pb[j] = xor_bits(PB, G.nb, b0 + 4 * tx + j);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t pa = xor_bits(PA, G.mb, a0 + 4 * ty + i) ^ pt;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint32_t v = PACK ? (acc[i][j >> 1] >> (16 * (j & 1))) & 0xFFFFu : acc[i][j];
            arena[G.po + (pa ^ pb[j])] = min(v, inf);
        }
    }
}

template <bool PACK>
static void launch_gemm(const TGemm &G, const uint32_t *gmaps, uint32_t *A, uint32_t inf, cudaStream_t s) {
    const dim3 grid(1u << (G.nb - 6), 1u << (G.mb - 6), 1u << G.kb);
    if (G.F >= 5) k_tree_gemm<PACK, 32><<<grid, 256, 0, s>>>(G, gmaps, A, inf);
    else if (G.F == 4) k_tree_gemm<PACK, 16><<<grid, 256, 0, s>>>(G, gmaps, A, inf);
    else if (G.F == 3) k_tree_gemm<PACK, 8><<<grid, 256, 0, s>>>(G, gmaps, A, inf);
    else k_tree_gemm<PACK, 4><<<grid, 256, 0, s>>>(G, gmaps, A, inf);
}

// ---------------------------------------------------------------- reference per-call entry points
template <typename T>
__device__ __forceinline__ void atomic_min_t(T *p, uint64_t v);
template <>
__device__ __forceinline__ void atomic_min_t<uint64_t>(uint64_t *p, uint64_t v) {
    atomicMin(reinterpret_cast<unsigned long long *>(p), (unsigned long long)v);
}
template <>
__device__ __forceinline__ void atomic_min_t<uint32_t>(uint32_t *p, uint64_t v) {
    atomicMin(p, (uint32_t)v);
}
// sub-word minimum through a compare-and-swap of the aligned word (each failed swap means another
// thread changed the word, so the loop ends; bounded all the same)
template <typename T>
__device__ __forceinline__ void atomic_min_sub(T *p, uint64_t v, int *err) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(p);
    uint32_t *w = reinterpret_cast<uint32_t *>(a & ~(uintptr_t)3);
    const int sh = (int)(a & 3) * 8;
    const uint32_t mask = (sizeof(T) == 1 ? 0xFFu : 0xFFFFu) << sh;
    uint32_t old = *w;
    for (int it = 0; it < (1 << 20); it++) {
        const uint32_t cur = (old & mask) >> sh;
        if (v >= cur) return;
        const uint32_t nw = (old & ~mask) | ((uint32_t)v << sh);
        const uint32_t got = atomicCAS(w, old, nw);
        if (got == old) return;
        old = got;
    }
    *err = 1;
}
struct RefMaps { uint64_t l[64], r[64]; };

template <typename T>
__global__ void k_tree_join_ref(const T *left, const T *right, T *out, const __grid_constant__ RefMaps mp,
                                unsigned parent_bits, uint64_t start, uint64_t stop, uint64_t inf, int *err) {
    const uint64_t i = start + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= stop) return;
    const uint64_t g = i ^ (i >> 1);
    uint64_t li = 0, ri = 0;
    for (uint64_t y = g; y; y &= y - 1) {
        const int b = __ffsll((long long)y) - 1;
        li ^= mp.l[b];
        ri ^= mp.r[b];
    }
    const uint64_t pi = parent_bits >= 64 ? g : (g & ((1ull << parent_bits) - 1ull));
    const uint64_t a = left[li], b = right[ri];
    if (a < inf && b < inf && a <= inf - b) {
        if constexpr (sizeof(T) >= 4) atomic_min_t<T>(out + pi, a + b);
        else atomic_min_sub<T>(out + pi, a + b, err);
    }
}

// forward overlapping copy in one block: tiles of at most `gap` bytes, each read completely
// before it is written
__global__ void k_tree_move(uint8_t *dst, const uint8_t *src, uint64_t bytes, uint64_t gap, int backward) {
    const uint64_t cap = (uint64_t)blockDim.x * 4, tile = gap < cap ? gap : cap;
    for (uint64_t done = 0; done < bytes; done += tile) {
        const uint64_t n = min(tile, bytes - done);
        const uint64_t base = backward ? bytes - done - n : done;
        uint8_t v[4];
        for (int k = 0; k < 4; k++) {
            const uint64_t e = (uint64_t)k * blockDim.x + threadIdx.x;
            if (e < n) v[k] = src[base + e];
        }
        __syncthreads();
        for (int k = 0; k < 4; k++) {
            const uint64_t e = (uint64_t)k * blockDim.x + threadIdx.x;
            if (e < n) dst[base + e] = v[k];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- plan
struct TreeStep {
    int kind;              // 0: k_tree_small over heights [h0, h1); 1: fill + joins of height h0
    int h0, h1;
    int64_t j0, nj, blocks, f0, nf, fill_blocks;
    std::vector<int64_t> gemms;   // block-product joins of this height (indexes into TreePlan::hg)
};

struct TreePlan {
    int64_t nleaves = 0, njoins = 0, nmaps = 0, arena = 0, root = 0, nwords = 0, pairs = 0;
    int nheights = 0;
    int64_t *d_leaves = nullptr, *d_lvl = nullptr;
    TJoin *d_joins = nullptr;
    TFill *d_fills = nullptr;
    uint32_t *d_maps = nullptr;
    uint64_t *d_target = nullptr;
    uint32_t *h_val = nullptr;      // pinned
    uint32_t *d_gmaps = nullptr;
    std::vector<TGemm> hg;
    std::vector<TreeStep> steps;
    int launches = 0;
};

static void tree_plan_release(TreePlan *T) {
    if (!T) return;
    cudaFree(T->d_leaves);
    cudaFree(T->d_lvl);
    cudaFree(T->d_joins);
    cudaFree(T->d_fills);
    cudaFree(T->d_maps);
    cudaFree(T->d_gmaps);
    cudaFree(T->d_target);
    if (T->h_val) cudaFreeHost(T->h_val);
    delete T;
}

}  // namespace tg

using namespace tg;

extern "C" {

// Whole-tree plan.  leaves: nleaves rows (offset, size 1|2, column, nonzero); joins: njoins rows
// (lo, ro, po, P, F, height, mapoff, 0) in nondecreasing height (heights 1, 2, ...); maps: for each
// generator (left state, right state) as uint32, generator i of a join at maps[2 * (mapoff + i)];
// arena: uint32 entries of the arena the plan's offsets address; root: offset of the root table;
// ncols: column count (the target representative has ceil(ncols / 64) words).
// small_pairs: heights of at most this many pairs run in the single-block kernel (< 0: 2^15);
// rbits: pairs per thread 2^min(F, rbits) in the join kernel (< 0: enough threads for the GPU).
// gemm: ngemm rows (join, F, mb, nb, kb, mapoff): joins run as min-plus block products, with their
// DL, DR, DT, PA, PB, PT vectors (uint32) at gmaps[mapoff]; a row needs F >= 2, 6 <= mb, nb <= 21,
// kb <= 16 and the join's F, parent rank and children's ranks to match.
void *tg_tree_plan(const int64_t *leaves, int64_t nleaves, const int64_t *joins, int64_t njoins,
                   const uint32_t *maps, int64_t nmaps, const int64_t *gemm, int64_t ngemm, const uint32_t *gmaps,
                   int64_t ngmaps, int64_t arena, int64_t root, int64_t ncols, int64_t small_pairs, int rbits,
                   int *status) {
    if (small_pairs < 0) small_pairs = TR_SMALL_PAIRS;
    if (ngemm < 0 || ngmaps < 0 || (ngemm && (!gemm || !gmaps))) {
        if (status) *status = set_error(TG_ERR_ARG, "bad tree gemm rows");
        return nullptr;
    }
    int st = TG_OK;
    TreePlan *T = nullptr;
    if (nleaves < 0 || njoins < 0 || nmaps < 0 || arena < 1 || root < 0 || root >= arena || ncols < 0 ||
        (nleaves && !leaves) || (njoins && !joins) || (nmaps && !maps)) {
        if (status) *status = set_error(TG_ERR_ARG, "bad tree plan");
        return nullptr;
    }
    T = new TreePlan();
    T->nleaves = nleaves;
    T->njoins = njoins;
    T->nmaps = nmaps;
    T->arena = arena;
    T->root = root;
    T->nwords = std::max<int64_t>(1, (ncols + 63) / 64);
    // every table a leaf or a join can address lies inside the arena: a join reads left states up to
    // the smear of the OR of its left maps (and the same for the right), writes 2^P parent entries
    for (int64_t i = 0; i < nleaves && st == TG_OK; i++) {
        const int64_t *r = leaves + 4 * i;
        if (r[0] < 0 || (r[1] != 1 && r[1] != 2) || r[0] + r[1] > arena || r[2] < 0 || r[2] >= ncols)
            st = set_error(TG_ERR_ARG, "bad tree leaf row");
    }
    for (int64_t j = 0; j < njoins && st == TG_OK; j++) {
        const int64_t *r = joins + 8 * j;
        const int64_t J = r[3] + r[4];
        if (J < 0 || J > TR_MAXJ || r[6] < 0 || r[6] + J > nmaps) continue;      // rejected below
        uint64_t ol = 0, orr = 0;
        for (int64_t g = 0; g < J; g++) { ol |= maps[2 * (r[6] + g)]; orr |= maps[2 * (r[6] + g) + 1]; }
        auto span = [](uint64_t v) -> int64_t { int64_t s = 1; while (v) { s <<= 1; v >>= 1; } return s; };
        if (r[0] < 0 || r[1] < 0 || r[0] + span(ol) > arena || r[1] + span(orr) > arena)
            st = set_error(TG_ERR_ARG, "tree join reads outside the arena");
    }
    std::vector<TJoin> hj((size_t)njoins);
    std::vector<int64_t> lvl;       // lvl[h] = first join of height h (heights from 1; lvl[0] unused)
    int hmax = 0;
    for (int64_t j = 0; j < njoins && st == TG_OK; j++) {
        const int64_t *r = joins + 8 * j;
        const int P = (int)r[3], F = (int)r[4], h = (int)r[5];
        if (P < 0 || F < 0 || P + F > TR_MAXJ || P > 32 || h < 1 || h < hmax || r[6] < 0 || r[6] + P + F > nmaps ||
            r[0] < 0 || r[1] < 0 || r[2] < 0 || r[2] + (1ll << P) > arena)
            st = set_error(TG_ERR_ARG, "bad tree join row");
        else {
            while (hmax < h) { lvl.resize((size_t)h + 1, j); hmax++; }
            hj[j].lo = r[0]; hj[j].ro = r[1]; hj[j].po = r[2];
            hj[j].P = P; hj[j].F = F; hj[j].mapoff = (int32_t)r[6];
            // pairs per thread: enough threads for the whole GPU, at most 2^11 pairs per thread
            const int J = P + F;
            hj[j].R = rbits >= 0 ? std::min(F, rbits) : std::min(F, std::max(std::min(F, 6), J - 19));
            // F >= 5: warp mode, a warp per (parent, chunk of 2^R pairs); at least 5 + 1 bits, at most
            // 2^11 pairs per lane, enough warps for the GPU
            hj[j].W = F >= 5 ? 1 : 0;
            hj[j].pad = 0;
            if (hj[j].W)
                hj[j].R = rbits >= 0 ? std::min(F, std::max(5, rbits))
                                     : std::min(F, std::max(5 + std::min(F - 5, 6), std::min(J - 14, 16)));
            else if (rbits < 0 && F <= 4 && P >= 14) {
                // mode 2: lane groups of 2^F lanes; R holds the parents walked per thread (up to 16,
                // keeping >= 2^14 groups)
                hj[j].W = 2;
                hj[j].R = std::min(4, P - 14);
            }
            T->pairs += 1ll << J;
        }
    }
    lvl.resize((size_t)hmax + 2, njoins);
    lvl[(size_t)hmax + 1] = njoins;
    T->nheights = hmax;
    // block-product joins: checked against the join rows and the arena, then taken out of the
    // join kernel's grid
    std::vector<int> gemm_of((size_t)njoins, -1);
    for (int64_t g = 0; g < ngemm && st == TG_OK; g++) {
        const int64_t *r = gemm + 6 * g;
        const int64_t j = r[0], F = r[1], mb = r[2], nb = r[3], kb = r[4], mo = r[5];
        if (j < 0 || j >= njoins || gemm_of[j] >= 0 || F < 2 || F > 30 || mb < 6 || mb > 21 || nb < 6 || nb > 21 ||
            kb < 0 || kb > 16 || mo < 0 || mo + 2 * (mb + nb + kb) > ngmaps || hj[j].F != F ||
            hj[j].P != mb + nb + kb) {
            st = set_error(TG_ERR_ARG, "bad tree gemm row");
            break;
        }
        const int64_t lsz = 1ll << (mb + F), rsz = 1ll << (nb + F);
        if (hj[j].lo + lsz > arena || hj[j].ro + rsz > arena || (hj[j].lo & 7) || (hj[j].ro & 7))
            st = set_error(TG_ERR_ARG, "tree gemm reads outside the arena");
        for (int64_t k = 0; k < mb + nb + kb && st == TG_OK; k++) {       // offsets below 2^F, parents below 2^P
            if (gmaps[mo + k] >> F) st = set_error(TG_ERR_ARG, "tree gemm offset out of range");
            if (hj[j].P < 32 && (gmaps[mo + mb + nb + kb + k] >> hj[j].P)) st = set_error(TG_ERR_ARG, "tree gemm parent out of range");
        }
        TGemm G;
        G.lo = hj[j].lo; G.ro = hj[j].ro; G.po = hj[j].po;
        G.F = (int32_t)F; G.mb = (int32_t)mb; G.nb = (int32_t)nb; G.kb = (int32_t)kb;
        G.mapoff = (int32_t)mo; G.pad = 0;
        gemm_of[j] = (int)T->hg.size();
        T->hg.push_back(G);
    }
    // steps: runs of small heights in one block, the others one launch each
    std::vector<TFill> fills;
    int64_t fill_block = 0;
    for (int h = 1; h <= hmax && st == TG_OK; h++) {
        int64_t pairs = 0;
        for (int64_t j = lvl[h]; j < lvl[h + 1]; j++) pairs += 1ll << (hj[j].P + hj[j].F);
        if (pairs <= small_pairs && lvl[h + 1] - lvl[h] <= 4) {     // a chain: one block, no launch per height
            for (int64_t j = lvl[h]; j < lvl[h + 1]; j++) gemm_of[j] = -1;    // tiny: the single-block kernel
            if (!T->steps.empty() && T->steps.back().kind == 0 && T->steps.back().h1 == h) T->steps.back().h1 = h + 1;
            else { TreeStep s{}; s.kind = 0; s.h0 = h; s.h1 = h + 1; T->steps.push_back(s); }
            continue;
        }
        TreeStep s{};
        s.kind = 1; s.h0 = h; s.h1 = h + 1; s.j0 = lvl[h]; s.nj = lvl[h + 1] - lvl[h];
        s.f0 = (int64_t)fills.size();
        fill_block = 0;
        int64_t blocks = 0;
        for (int64_t j = lvl[h]; j < lvl[h + 1]; j++) {
            TJoin &d = hj[j];
            d.block0 = blocks;
            if (gemm_of[j] >= 0) { s.gemms.push_back(gemm_of[j]); continue; }   // no blocks in k_tree_join
            const int tb = d.W == 2 ? d.P - d.R + d.F : d.P + d.F - d.R + (d.W ? 5 : 0);
            blocks += (int64_t)(((1ull << tb) + TR_BS - 1) / TR_BS);
            if (d.W != 2 && d.F > d.R) {
                const int64_t size = 1ll << d.P;
                fills.push_back(TFill{d.po, size, fill_block});
                fill_block += (size + TR_BS * 8 - 1) / (TR_BS * 8);
            }
        }
        if (blocks > 0x7FFFFFFFll || fill_block > 0x7FFFFFFFll) st = set_error(TG_ERR_TOO_BIG, "tree join grid");
        s.blocks = blocks;
        s.nf = (int64_t)fills.size() - s.f0;
        s.fill_blocks = fill_block;
        T->steps.push_back(s);
    }
    // fills are indexed per step (block0 restarts at every step): keep them contiguous per step
    if (st == TG_OK) {
        auto alloc = [&](void **p, size_t n) {
            if (st) return;
            if (cudaMalloc(p, std::max<size_t>(n, 8)) != cudaSuccess) {
                cudaGetLastError();
                st = set_error(TG_ERR_NOMEM, "tree plan buffers");
            }
        };
        alloc((void **)&T->d_leaves, (size_t)nleaves * 32);
        alloc((void **)&T->d_joins, hj.size() * sizeof(TJoin));
        alloc((void **)&T->d_lvl, lvl.size() * 8);
        alloc((void **)&T->d_fills, fills.size() * sizeof(TFill));
        alloc((void **)&T->d_maps, (size_t)nmaps * 8);
        alloc((void **)&T->d_target, (size_t)T->nwords * 8);
        alloc((void **)&T->d_gmaps, (size_t)std::max<int64_t>(ngmaps, 1) * 4);
        if (!st && cudaMallocHost(&T->h_val, 64) != cudaSuccess) {
            cudaGetLastError();
            T->h_val = nullptr;
            st = set_error(TG_ERR_NOMEM, "pinned result word");
        }
        if (!st && nleaves) st = cuda_check(cudaMemcpy(T->d_leaves, leaves, (size_t)nleaves * 32, cudaMemcpyHostToDevice), "leaves");
        if (!st && njoins) st = cuda_check(cudaMemcpy(T->d_joins, hj.data(), hj.size() * sizeof(TJoin), cudaMemcpyHostToDevice), "joins");
        if (!st) st = cuda_check(cudaMemcpy(T->d_lvl, lvl.data(), lvl.size() * 8, cudaMemcpyHostToDevice), "heights");
        if (!st && !fills.empty()) st = cuda_check(cudaMemcpy(T->d_fills, fills.data(), fills.size() * sizeof(TFill), cudaMemcpyHostToDevice), "fills");
        if (!st && nmaps) st = cuda_check(cudaMemcpy(T->d_maps, maps, (size_t)nmaps * 8, cudaMemcpyHostToDevice), "maps");
        if (!st && ngmaps) st = cuda_check(cudaMemcpy(T->d_gmaps, gmaps, (size_t)ngmaps * 4, cudaMemcpyHostToDevice), "gemm maps");
    }
    if (st) {
        tree_plan_release(T);
        T = nullptr;
    } else {
        T->launches = 1 + (nleaves ? 1 : 0);
        for (const TreeStep &s : T->steps)
            T->launches += s.kind == 0 ? 1 : (s.blocks ? 1 : 0) + (s.nf ? 1 : 0) + (int)s.gemms.size();
    }
    if (status) *status = st;
    return T;
}

// info: heights, steps, launches per run, pairs (join work), arena entries, nleaves, njoins, small steps,
// block-product joins
int tg_tree_plan_info(void *p, int64_t *info, int n) {
    TreePlan *T = static_cast<TreePlan *>(p);
    if (!T || !info) return set_error(TG_ERR_ARG, "null tree plan");
    int64_t small = 0;
    for (const TreeStep &s : T->steps) small += s.kind == 0;
    const int64_t v[9] = {T->nheights, (int64_t)T->steps.size(), T->launches, T->pairs, T->arena, T->nleaves,
                          T->njoins, small, (int64_t)T->hg.size()};
    for (int i = 0; i < n && i < 9; i++) info[i] = v[i];
    return TG_OK;
}

// Run the plan for one target: `target` (HOST, ceil(ncols / 64) words) is the bit vector of a
// particular solution e0 of M e0 = target; arena (DEVICE, uint32 entries); *value = the root entry
// (INF = `inf` when the target has no finite solution, which a consistent system never gives).
int tg_tree_run(void *p, void *arena, const uint64_t *target, uint32_t inf, uint32_t *value, void *stream) {
    TreePlan *T = static_cast<TreePlan *>(p);
    if (!T || !arena || !target || !value) return set_error(TG_ERR_ARG, "bad tree run");
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t *A = static_cast<uint32_t *>(arena);
    int e = cuda_check(cudaMemcpyAsync(T->d_target, target, (size_t)T->nwords * 8, cudaMemcpyHostToDevice, s),
                       "target");
    if (e) return e;
    if (T->nleaves)
        k_tree_leaves<<<(unsigned)((T->nleaves + 255) / 256), 256, 0, s>>>(T->d_leaves, T->nleaves, T->d_target, A);
    for (const TreeStep &st : T->steps) {
        if (st.kind == 0) {
            k_tree_small<<<1, 1024, 0, s>>>(T->d_joins, T->d_lvl, st.h0, st.h1, T->d_maps, A, inf);
        } else {
            if (st.nf) k_tree_fill<<<(unsigned)st.fill_blocks, TR_BS, 0, s>>>(T->d_fills + st.f0, (int)st.nf, A, inf);
            if (st.blocks)
                k_tree_join<<<(unsigned)st.blocks, TR_BS, 0, s>>>(T->d_joins + st.j0, (int)st.nj, T->d_maps, A, inf);
            for (int64_t g : st.gemms) {
                const TGemm &G = T->hg[(size_t)g];
                if (inf < 32768u) launch_gemm<true>(G, T->d_gmaps, A, inf, s);
                else launch_gemm<false>(G, T->d_gmaps, A, inf, s);
            }
        }
    }
    e = cuda_check(cudaGetLastError(), "tree launches");
    if (e) return e;
    e = cuda_check(cudaMemcpyAsync(T->h_val, A + T->root, 4, cudaMemcpyDeviceToHost, s), "root");
    if (!e) e = cuda_check(cudaStreamSynchronize(s), "tree run");
    if (!e) *value = T->h_val[0];
    return e;
}

void tg_tree_plan_free(void *p) { tree_plan_release(static_cast<TreePlan *>(p)); }

// cdist/tree_dp.c:13-39 tree_join_u*: the pairs i in [start, stop) of a join in Gray order on DEVICE
// tables; lm / rm are HOST arrays of `generators` (<= 64) maps; out[parent] = min(out[parent], a + b)
// for finite a, b with a + b <= infinity (the sum of the reference's `a <= infinity - b` test).
#define TREE_JOIN_REF(T, NAME)                                                                              \
int NAME(const void *left, const void *right, void *out, const uint64_t *lm, const uint64_t *rm,             \
         unsigned parent_bits, unsigned generators, uint64_t start, uint64_t stop, uint64_t infinity) {      \
    if (!left || !right || !out || generators > 64 || parent_bits > generators || (generators && (!lm || !rm))) \
        return set_error(TG_ERR_ARG, "bad tree join");                                                      \
    if (stop <= start) return TG_OK;                                                                        \
    RefMaps mp;                                                                                             \
    memset(&mp, 0, sizeof(mp));                                                                             \
    for (unsigned i = 0; i < generators; i++) { mp.l[i] = lm[i]; mp.r[i] = rm[i]; }                        \
    int *err = nullptr;                                                                                     \
    if (cudaMalloc(&err, 4) != cudaSuccess) { cudaGetLastError(); return set_error(TG_ERR_NOMEM, "flag"); } \
    cudaMemsetAsync(err, 0, 4, cur_stream());                                                               \
    const uint64_t n = stop - start;                                                                        \
    const uint64_t per = 256ull * 65535ull * 1024ull;                                                       \
    for (uint64_t b = 0; b < n; b += per) {                                                                 \
        const uint64_t m = std::min(per, n - b);                                                            \
        k_tree_join_ref<T><<<(unsigned)((m + 255) / 256), 256, 0, cur_stream()>>>(                         \
            (const T *)left, (const T *)right, (T *)out, mp, parent_bits, start + b, start + b + m,         \
            infinity, err);                                                                                 \
    }                                                                                                       \
    int h = 0;                                                                                              \
    int e = cuda_check(cudaMemcpyAsync(&h, err, 4, cudaMemcpyDeviceToHost, cur_stream()), "tree join");     \
    if (!e) e = cuda_check(cudaStreamSynchronize(cur_stream()), "tree join");                               \
    cudaFree(err);                                                                                          \
    if (!e && h) e = set_error(TG_ERR_TIMEOUT, "tree join: compare-and-swap did not settle");               \
    return e;                                                                                               \
}
TREE_JOIN_REF(uint8_t, tree_join_u8)
TREE_JOIN_REF(uint16_t, tree_join_u16)
TREE_JOIN_REF(uint32_t, tree_join_u32)
TREE_JOIN_REF(uint64_t, tree_join_u64)

// cdist/tree_dp.c:45-50 tree_move: memmove between DEVICE addresses (regions may overlap)
int tree_move(void *destination, const void *source, size_t bytes) {
    if (!bytes || destination == source) return TG_OK;
    if (!destination || !source) return set_error(TG_ERR_ARG, "bad tree move");
    uint8_t *d = static_cast<uint8_t *>(destination);
    const uint8_t *s = static_cast<const uint8_t *>(source);
    const bool overlap = d < s + bytes && s < d + bytes;
    if (!overlap) return cuda_check(cudaMemcpyAsync(d, s, bytes, cudaMemcpyDeviceToDevice, cur_stream()), "tree move");
    const uint64_t gap = d < s ? (uint64_t)(s - d) : (uint64_t)(d - s);
    k_tree_move<<<1, 1024, 0, cur_stream()>>>(d, s, bytes, gap, d > s ? 1 : 0);
    return cuda_check(cudaGetLastError(), "tree move");
}

}  // extern "C"
