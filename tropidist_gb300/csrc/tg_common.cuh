// Shared device helpers of libtropigpu (sm_103a).
//
// Tables hold minimum weights as uint8 (INF = 255) or uint16 (INF = 65535).  The min-plus rule of
// one column is  T[s] = min(T[s], sat(T[s ^ h] + w))  with saturation at INF.  Because every entry
// is <= INF, min(a, sat(b + w)) == min(a, b + w) whenever b + w is computed without wrapping, so the
// kernels widen entries by one size class (u8 -> u16 lanes, u16 -> u32 lanes) and use the DPX
// add-then-min instructions, which need no saturation step at all.
#pragma once
#include <cstdint>
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#define TG_INF8 255u
#define TG_INF16 65535u

// status codes shared by every C-ABI entry point
#define TG_OK 0
#define TG_ERR_ARG -1          // bad argument (sizes, masks, op stream)
#define TG_ERR_CUDA -2         // a CUDA runtime call failed (tg_last_error has the text)
#define TG_ERR_NOMEM -3        // a device allocation failed
#define TG_ERR_TOO_BIG -4      // a size beyond a documented maximum
#define TG_ERR_TIMEOUT -5      // a bounded device wait ran out
#define TG_ERR_STATE -6        // called in the wrong state (e.g. a freed handle)

namespace tg {

template <typename E> struct Entry;
template <> struct Entry<uint8_t> {
    static constexpr int CB = 4;                 // log2 entries per 16-byte chunk
    static constexpr uint32_t INF = TG_INF8;
    static constexpr uint32_t INF_WORD = 0xFFFFFFFFu;
};
template <> struct Entry<uint16_t> {
    static constexpr int CB = 3;
    static constexpr uint32_t INF = TG_INF16;
    static constexpr uint32_t INF_WORD = 0xFFFFFFFFu;
};

// per byte: min(a, b + w), for packed uint8 words (w <= 255 - 0, no wrap in u16 lanes)
__device__ __forceinline__ uint32_t minplus_u8x4(uint32_t a, uint32_t b, uint32_t w2) {
    uint32_t alo = __byte_perm(a, 0u, 0x4140), ahi = __byte_perm(a, 0u, 0x4342);
    uint32_t blo = __byte_perm(b, 0u, 0x4140), bhi = __byte_perm(b, 0u, 0x4342);
    uint32_t rlo = __viaddmin_u16x2(blo, w2, alo);
    uint32_t rhi = __viaddmin_u16x2(bhi, w2, ahi);
    return __byte_perm(rlo, rhi, 0x6420);
}

// both directions of a pair of packed uint8 words: a' = min(a, b + w), b' = min(b, a + w)
__device__ __forceinline__ void minplus_pair_u8x4(uint32_t &a, uint32_t &b, uint32_t w2) {
    uint32_t alo = __byte_perm(a, 0u, 0x4140), ahi = __byte_perm(a, 0u, 0x4342);
    uint32_t blo = __byte_perm(b, 0u, 0x4140), bhi = __byte_perm(b, 0u, 0x4342);
    uint32_t ralo = __viaddmin_u16x2(blo, w2, alo), rahi = __viaddmin_u16x2(bhi, w2, ahi);
    uint32_t rblo = __viaddmin_u16x2(alo, w2, blo), rbhi = __viaddmin_u16x2(ahi, w2, bhi);
    a = __byte_perm(ralo, rahi, 0x6420);
    b = __byte_perm(rblo, rbhi, 0x6420);
}

// per halfword: min(a, b + w) for packed uint16 words (computed in 32-bit lanes: no wrap)
__device__ __forceinline__ uint32_t minplus_u16x2(uint32_t a, uint32_t b, uint32_t w) {
    uint32_t lo = min(a & 0xFFFFu, (b & 0xFFFFu) + w);
    uint32_t hi = min(a >> 16, (b >> 16) + w);
    return lo | (hi << 16);
}

// byte permutation of a word: byte i <- byte i ^ x (x < 4)
__device__ __forceinline__ uint32_t xor_bytes(uint32_t v, uint32_t x) {
    const uint32_t sel = (0u ^ x) | ((1u ^ x) << 4) | ((2u ^ x) << 8) | ((3u ^ x) << 12);
    return __byte_perm(v, 0u, sel);
}

// A counter increment shared by the lanes that reach it together: one atomic per group of
// converged lanes (same-address atomics from every lane serialise in one L2 slice).  Returns this
// lane's value of the counter before the increment.
__device__ __forceinline__ unsigned long long agg_inc(unsigned long long *ctr) {
    namespace cg = cooperative_groups;
    const cg::coalesced_group g = cg::coalesced_threads();
    unsigned long long base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(ctr, (unsigned long long)g.size());
    return g.shfl(base, 0) + g.thread_rank();
}

// Output slots for the threads of a block that want them, in up to two counters at once, with one
// atomic per block, call and counter.  Every thread of the block must make the call the same
// number of times (wants may be false), with the same phase variable (it alternates two sets of
// shared slots, so that one call needs two barriers); blockDim.x a multiple of 32, at most 1024.
// ja / jb: this thread's slots (meaningless where it did not want one); cb may be null.
__device__ __forceinline__ void block_claim2(unsigned &phase, unsigned long long *ca, bool wa, unsigned long long *cb,
                                             bool wb, unsigned long long &ja, unsigned long long &jb) {
    __shared__ unsigned s_off[2][2][32];
    __shared__ unsigned long long s_base[2][2];
    const unsigned buf = phase & 1u;
    phase++;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const unsigned balA = __ballot_sync(0xffffffffu, wa), balB = __ballot_sync(0xffffffffu, wb);
    if (lane == 0) {
        s_off[buf][0][warp] = __popc(balA);
        s_off[buf][1][warp] = __popc(balB);
    }
    __syncthreads();
    if (warp == 0) {
        const unsigned nw = blockDim.x >> 5;
        const unsigned ca0 = lane < nw ? s_off[buf][0][lane] : 0u, cb0 = lane < nw ? s_off[buf][1][lane] : 0u;
        unsigned xa = ca0, xb = cb0;
        for (unsigned off = 1; off < 32; off <<= 1) {
            const unsigned ya = __shfl_up_sync(0xffffffffu, xa, off), yb = __shfl_up_sync(0xffffffffu, xb, off);
            if (lane >= off) {
                xa += ya;
                xb += yb;
            }
        }
        const unsigned ta = __shfl_sync(0xffffffffu, xa, 31), tb = __shfl_sync(0xffffffffu, xb, 31);
        if (lane < nw) {
            s_off[buf][0][lane] = xa - ca0;
            s_off[buf][1][lane] = xb - cb0;
        }
        if (lane == 0) {
            s_base[buf][0] = ta ? atomicAdd(ca, (unsigned long long)ta) : 0ull;
            s_base[buf][1] = (tb && cb) ? atomicAdd(cb, (unsigned long long)tb) : 0ull;
        }
    }
    __syncthreads();
    const unsigned below = (1u << lane) - 1u;
    ja = s_base[buf][0] + s_off[buf][0][warp] + __popc(balA & below);
    jb = s_base[buf][1] + s_off[buf][1][warp] + __popc(balB & below);
}

// block_claim2 for counts: this thread wants na slots of counter ca and nb of cb (an inclusive
// scan over the warp, then over the warps); ja / jb: the first of its slots.  Same rules as
// block_claim2 (every thread calls, the same number of times, one phase variable).
__device__ __forceinline__ void block_claim2_n(unsigned &phase, unsigned long long *ca, unsigned na,
                                               unsigned long long *cb, unsigned nb, unsigned long long &ja,
                                               unsigned long long &jb) {
    __shared__ unsigned s_w[2][2][32];
    __shared__ unsigned long long s_b[2][2];
    const unsigned buf = phase & 1u;
    phase++;
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned xa = na, xb = nb;
    for (unsigned off = 1; off < 32; off <<= 1) {
        const unsigned ya = __shfl_up_sync(0xffffffffu, xa, off), yb = __shfl_up_sync(0xffffffffu, xb, off);
        if (lane >= off) {
            xa += ya;
            xb += yb;
        }
    }
    if (lane == 31) {
        s_w[buf][0][warp] = xa;
        s_w[buf][1][warp] = xb;
    }
    __syncthreads();
    if (warp == 0) {
        const unsigned nw = blockDim.x >> 5;
        const unsigned va = lane < nw ? s_w[buf][0][lane] : 0u, vb = lane < nw ? s_w[buf][1][lane] : 0u;
        unsigned za = va, zb = vb;
        for (unsigned off = 1; off < 32; off <<= 1) {
            const unsigned ya = __shfl_up_sync(0xffffffffu, za, off), yb = __shfl_up_sync(0xffffffffu, zb, off);
            if (lane >= off) {
                za += ya;
                zb += yb;
            }
        }
        const unsigned ta = __shfl_sync(0xffffffffu, za, 31), tb = __shfl_sync(0xffffffffu, zb, 31);
        if (lane < nw) {
            s_w[buf][0][lane] = za - va;
            s_w[buf][1][lane] = zb - vb;
        }
        if (lane == 0) {
            s_b[buf][0] = ta ? atomicAdd(ca, (unsigned long long)ta) : 0ull;
            s_b[buf][1] = (tb && cb) ? atomicAdd(cb, (unsigned long long)tb) : 0ull;
        }
    }
    __syncthreads();
    ja = s_b[buf][0] + s_w[buf][0][warp] + (xa - na);
    jb = s_b[buf][1] + s_w[buf][1][warp] + (xb - nb);
}

__device__ __forceinline__ unsigned long long block_claim(unsigned &phase, unsigned long long *ctr, bool want) {
    unsigned long long j, unused;
    block_claim2(phase, ctr, want, nullptr, false, j, unused);
    return j;
}

// Add every thread's count to a counter, one atomic per group of converged lanes (at kernel end).
__device__ __forceinline__ void agg_add(unsigned long long *ctr, unsigned long long x) {
    namespace cg = cooperative_groups;
    const cg::coalesced_group g = cg::coalesced_threads();
    for (unsigned off = 1; off < g.size(); off <<= 1) {
        const unsigned long long y = g.shfl_down(x, off);
        if (g.thread_rank() + off < g.size()) x += y;
    }
    if (g.thread_rank() == 0 && x) atomicAdd(ctr, x);
}

// 16-byte chunk as 4 words
struct Chunk { uint32_t w[4]; };

__device__ __forceinline__ Chunk ld_chunk(const void *p) {
    uint4 v = *reinterpret_cast<const uint4 *>(p);
    Chunk c; c.w[0] = v.x; c.w[1] = v.y; c.w[2] = v.z; c.w[3] = v.w; return c;
}
__device__ __forceinline__ void st_chunk(void *p, const Chunk &c) {
    *reinterpret_cast<uint4 *>(p) = make_uint4(c.w[0], c.w[1], c.w[2], c.w[3]);
}
__device__ __forceinline__ Chunk ld_chunk_cg(const void *p) {   // through L2 (written by other SMs)
    uint4 v = __ldcg(reinterpret_cast<const uint4 *>(p));
    Chunk c; c.w[0] = v.x; c.w[1] = v.y; c.w[2] = v.z; c.w[3] = v.w; return c;
}
__device__ __forceinline__ Chunk ldg_chunk(const void *p) {
    uint4 v = __ldcs(reinterpret_cast<const uint4 *>(p));   // streamed once: evict-first
    Chunk c; c.w[0] = v.x; c.w[1] = v.y; c.w[2] = v.z; c.w[3] = v.w; return c;
}
__device__ __forceinline__ void stg_chunk(void *p, const Chunk &c) {
    __stcs(reinterpret_cast<uint4 *>(p), make_uint4(c.w[0], c.w[1], c.w[2], c.w[3]));
}

// word permutation of a chunk: word k <- word k ^ wx (selects, no dynamic register indexing)
__device__ __forceinline__ void chunk_xor_words(uint32_t &x0, uint32_t &x1, uint32_t &x2, uint32_t &x3, uint32_t wx) {
    uint32_t t;
    if (wx & 1u) { t = x0; x0 = x1; x1 = t; t = x2; x2 = x3; x3 = t; }
    if (wx & 2u) { t = x0; x0 = x2; x2 = t; t = x1; x1 = x3; x3 = t; }
}

// entry permutation inside a chunk: entry i <- entry i ^ m (m < entries per chunk)
template <typename E> __device__ __forceinline__ Chunk chunk_xor(const Chunk &c, uint32_t m);
template <> __device__ __forceinline__ Chunk chunk_xor<uint8_t>(const Chunk &c, uint32_t m) {
    uint32_t x0 = c.w[0], x1 = c.w[1], x2 = c.w[2], x3 = c.w[3];
    chunk_xor_words(x0, x1, x2, x3, m >> 2);
    const uint32_t bx = m & 3u;
    Chunk r;
    if (bx) {
        r.w[0] = xor_bytes(x0, bx); r.w[1] = xor_bytes(x1, bx); r.w[2] = xor_bytes(x2, bx); r.w[3] = xor_bytes(x3, bx);
    } else {
        r.w[0] = x0; r.w[1] = x1; r.w[2] = x2; r.w[3] = x3;
    }
    return r;
}
template <> __device__ __forceinline__ Chunk chunk_xor<uint16_t>(const Chunk &c, uint32_t m) {
    uint32_t x0 = c.w[0], x1 = c.w[1], x2 = c.w[2], x3 = c.w[3];
    chunk_xor_words(x0, x1, x2, x3, m >> 1);
    Chunk r;
    if (m & 1u) {
        r.w[0] = __byte_perm(x0, 0u, 0x1032); r.w[1] = __byte_perm(x1, 0u, 0x1032);
        r.w[2] = __byte_perm(x2, 0u, 0x1032); r.w[3] = __byte_perm(x3, 0u, 0x1032);
    } else {
        r.w[0] = x0; r.w[1] = x1; r.w[2] = x2; r.w[3] = x3;
    }
    return r;
}

// chunk-wise min-plus: a' = min(a, b + w) entrywise
template <typename E> __device__ __forceinline__ Chunk chunk_minplus(const Chunk &a, const Chunk &b, uint32_t w);
template <> __device__ __forceinline__ Chunk chunk_minplus<uint8_t>(const Chunk &a, const Chunk &b, uint32_t w) {
    Chunk r;
    const uint32_t w2 = w | (w << 16);
#pragma unroll
    for (int k = 0; k < 4; k++) r.w[k] = minplus_u8x4(a.w[k], b.w[k], w2);
    return r;
}
template <> __device__ __forceinline__ Chunk chunk_minplus<uint16_t>(const Chunk &a, const Chunk &b, uint32_t w) {
    Chunk r;
#pragma unroll
    for (int k = 0; k < 4; k++) r.w[k] = minplus_u16x2(a.w[k], b.w[k], w);
    return r;
}

// both directions at once on aligned chunks: a <- min(a, b + w), b <- min(b, a + w)
template <typename E> __device__ __forceinline__ void chunk_minplus_pair(Chunk &a, Chunk &b, uint32_t w);
template <> __device__ __forceinline__ void chunk_minplus_pair<uint8_t>(Chunk &a, Chunk &b, uint32_t w) {
    const uint32_t w2 = w | (w << 16);
#pragma unroll
    for (int k = 0; k < 4; k++) minplus_pair_u8x4(a.w[k], b.w[k], w2);
}
template <> __device__ __forceinline__ void chunk_minplus_pair<uint16_t>(Chunk &a, Chunk &b, uint32_t w) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
        uint32_t x = a.w[k], y = b.w[k];
        a.w[k] = minplus_u16x2(x, y, w);
        b.w[k] = minplus_u16x2(y, x, w);
    }
}

// asynchronous 16-byte global -> shared copies (L2 only)
__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait_group() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// scalar rule on one entry
template <typename E> __device__ __forceinline__ E minplus1(E a, E b, uint32_t w) {
    uint32_t x = (uint32_t)b + w;
    return (E)min((uint32_t)a, x);
}

// index with a zero bit inserted at position b
__device__ __forceinline__ uint32_t insert_zero(uint32_t p, int b) {
    uint32_t lo = p & ((1u << b) - 1u);
    return ((p ^ lo) << 1) | lo;
}
__device__ __forceinline__ uint64_t insert_zero64(uint64_t p, int b) {
    uint64_t lo = p & ((1ull << b) - 1ull);
    return ((p ^ lo) << 1) | lo;
}

}  // namespace tg
