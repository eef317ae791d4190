// Exact min-plus tree DP on the GPU (cdist/tree_dp.c:13-43, cdist/tree_dp.py:409-501).
//
// A binary tree over the columns has one table per node, indexed by the node's interface state;
// a join enumerates the 2^J compatible (left, right) state pairs of a node, J = P + F: generators
// 0..P-1 lift the parent's unit vectors, generators P..J-1 span the kernel of child addition.
// Pair x in [0, 2^J) has left state XOR(lmap[i] : bit i of x), right state XOR(rmap[i]) and parent
// x & (2^P - 1); the parent entry is the least left + right over its pairs (entries < INF =
// ncols + 1; a finite sum never reaches INF, since the two subtrees' columns are disjoint).
//
// Device tables are uint32 in one arena.  A tree plan (host-built) lists the leaves and the joins
// grouped by height: every join of one height runs in one launch, which is
//   - k_tree_small: one block runs a whole run of consecutive small heights (a few thousand
//     pairs each, e.g. the long spine of a comb tree) with a block barrier between heights;
//   - k_tree_fill + k_tree_join: each thread walks 2^R pairs of one parent in Gray order (R <= F;
//     inner 2^min(R,6) steps unrolled, so the generators sit in registers and all loads of a
//     thread are independent), keeps the least sum and, when a parent's pairs span threads,
//     reduces across the warp and commits with atomicMin into a table pre-filled with INF.
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
    int32_t P, F, R, mapoff;   // parent rank, kernel generators, pair bits per thread, maps index
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

__global__ void __launch_bounds__(TR_BS, 4) k_tree_join(const TJoin *joins, int nj, const uint32_t *maps,
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
    int kind;              // 0: k_tree_small over heights [h0, h1); 1: fill + join of height h0
    int h0, h1;
    int64_t j0, nj, blocks, f0, nf, fill_blocks;
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
void *tg_tree_plan(const int64_t *leaves, int64_t nleaves, const int64_t *joins, int64_t njoins,
                   const uint32_t *maps, int64_t nmaps, int64_t arena, int64_t root, int64_t ncols,
                   int64_t small_pairs, int rbits, int *status) {
    if (small_pairs < 0) small_pairs = TR_SMALL_PAIRS;
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
            T->pairs += 1ll << J;
        }
    }
    lvl.resize((size_t)hmax + 2, njoins);
    lvl[(size_t)hmax + 1] = njoins;
    T->nheights = hmax;
    // steps: runs of small heights in one block, the others one launch each
    std::vector<TFill> fills;
    int64_t fill_block = 0;
    for (int h = 1; h <= hmax && st == TG_OK; h++) {
        int64_t pairs = 0;
        for (int64_t j = lvl[h]; j < lvl[h + 1]; j++) pairs += 1ll << (hj[j].P + hj[j].F);
        if (pairs <= small_pairs) {
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
            blocks += (int64_t)(((1ull << (d.P + d.F - d.R)) + TR_BS - 1) / TR_BS);
            if (d.F > d.R) {
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
    }
    if (st) {
        tree_plan_release(T);
        T = nullptr;
    } else {
        T->launches = 1 + (nleaves ? 1 : 0);
        for (const TreeStep &s : T->steps) T->launches += s.kind == 0 ? 1 : 1 + (s.nf ? 1 : 0);
    }
    if (status) *status = st;
    return T;
}

// info: heights, steps, launches per run, pairs (join work), arena entries, nleaves, njoins, small steps
int tg_tree_plan_info(void *p, int64_t *info, int n) {
    TreePlan *T = static_cast<TreePlan *>(p);
    if (!T || !info) return set_error(TG_ERR_ARG, "null tree plan");
    int64_t small = 0;
    for (const TreeStep &s : T->steps) small += s.kind == 0;
    const int64_t v[8] = {T->nheights, (int64_t)T->steps.size(), T->launches, T->pairs, T->arena, T->nleaves,
                          T->njoins, small};
    for (int i = 0; i < n && i < 8; i++) info[i] = v[i];
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
            k_tree_join<<<(unsigned)st.blocks, TR_BS, 0, s>>>(T->d_joins + st.j0, (int)st.nj, T->d_maps, A, inf);
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
