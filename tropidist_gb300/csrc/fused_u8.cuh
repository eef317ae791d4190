// Register-resident update groups for uint8 tables (the inner loop of the fused tile pass).
//
// A group is a set of update ops of one pass whose chunk masks (mask >> 4: the part above the 16
// entries of a 16-byte chunk) span a subspace of dimension <= 3 of the tile's chunk index.  Let
// b0, b1, b2 be a reduced basis of that subspace extended to dimension 3, with pivot bits p0, p1,
// p2 (bit p_j set in b_j only).  The tile's chunks split into cosets {c0 ^ X[x] : x < 8}, X[x] =
// XOR of the b_j selected by the bits of x, c0 ranging over the chunk indices with zero pivot
// bits.  Every update of the group pairs chunks inside one coset, so a thread loads a whole coset
// (8 chunks = 128 entries) into registers, applies every update of the group there and writes it
// back: one shared-memory round trip per group instead of one per update.
//
// Register file: R[4 * x + k] holds word k (entries 4k .. 4k+3, packed bytes) of chunk x.  A group
// holds only updates without in-chunk bits (the scheduler keeps rows that are being updated out
// of the four in-chunk positions; the rare others run in shared memory), so an update with chunk
// coordinates y (b-basis) pairs chunk x with chunk x ^ y word for word; each word pair is widened
// to 16-bit lanes once for both directions (minplus_pair_u8x4).  y is dispatched through a switch
// to code unrolled by template recursion: every register index is a compile-time constant.
#pragma once
#include "tg_common.cuh"

namespace tg {

#define FP_MAXG 16

struct GroupDesc {
    uint32_t xoff[8];        // chunk offsets X[x] inside a coset
    uint8_t piv[3];          // pivot chunk bits, ascending
    uint8_t first, count;    // the group's codes: ucode[first .. first + count)
    uint8_t pad[3];
};

__device__ __forceinline__ uint32_t swap_halves(uint32_t v) { return __byte_perm(v, 0u, 0x1032); }

// widen a packed word (bytes e0..e3) to (e0, e2) and (e1, e3) halfword lanes, and back
__device__ __forceinline__ void unpack_eo(uint32_t w, uint32_t &e, uint32_t &o) {
    e = w & 0x00FF00FFu;
    o = __byte_perm(w, 0u, 0x4341);
}
__device__ __forceinline__ uint32_t pack_eo(uint32_t e, uint32_t o) { return e | (o << 8); }

// chunk-level update on packed words: chunk X (R[4X .. 4X+3]) pairs with chunk X ^ Y, unrolled
// by template recursion (every register index is a compile-time constant)
template <int Y, int X>
struct GrpPairs {
    static __device__ __forceinline__ void run(uint32_t (&R)[32], uint32_t w2) {
        if constexpr (X < (X ^ Y)) {
#pragma unroll
            for (int k = 0; k < 4; k++) minplus_pair_u8x4(R[4 * X + k], R[4 * (X ^ Y) + k], w2);
        }
        if constexpr (X < 7) GrpPairs<Y, X + 1>::run(R, w2);
    }
};

// y in 1..7: the update's chunk mask in the coset basis
__device__ __forceinline__ void grp_dispatch(uint32_t y, uint32_t (&R)[32], uint32_t w2) {
    switch (y) {
        case 1: GrpPairs<1, 0>::run(R, w2); break;
        case 2: GrpPairs<2, 0>::run(R, w2); break;
        case 3: GrpPairs<3, 0>::run(R, w2); break;
        case 4: GrpPairs<4, 0>::run(R, w2); break;
        case 5: GrpPairs<5, 0>::run(R, w2); break;
        case 6: GrpPairs<6, 0>::run(R, w2); break;
        case 7: GrpPairs<7, 0>::run(R, w2); break;
        default: break;
    }
}

// one group over a shared-memory tile of 2^d entries (chunks of 16 entries), all threads
template <int NT>
__device__ __forceinline__ void run_group(uint4 *TC, int d, const GroupDesc &g, const uint8_t *ucode,
                                          const uint8_t *uw) {
    const uint32_t ncos = 1u << (d - 4 - 3);
    const int p0 = g.piv[0], p1 = g.piv[1], p2 = g.piv[2];
    for (uint32_t k = threadIdx.x; k < ncos; k += NT) {
        // coset representative: k with zero bits inserted at the pivots (ascending)
        const uint32_t c0 = insert_zero(insert_zero(insert_zero(k, p0), p1), p2);
        uint32_t R[32];
#pragma unroll
        for (int x = 0; x < 8; x++) {
            const uint4 v = TC[c0 ^ g.xoff[x]];
            R[4 * x + 0] = v.x; R[4 * x + 1] = v.y; R[4 * x + 2] = v.z; R[4 * x + 3] = v.w;
        }
        for (int u = 0; u < g.count; u++) {
            const uint32_t w = uw[g.first + u];
            grp_dispatch(ucode[g.first + u], R, w | (w << 16));
        }
#pragma unroll
        for (int x = 0; x < 8; x++) TC[c0 ^ g.xoff[x]] = make_uint4(R[4 * x], R[4 * x + 1], R[4 * x + 2], R[4 * x + 3]);
    }
}

// output chunk of a pass that selects exactly one of the local bits 0..3 (bit s, target t):
// compacted entries 0..15 come from the 32 entries of chunks A (local bit 4 = 0) and B (= 1)
__device__ __forceinline__ uint4 gather_one_select(const uint4 &A, const uint4 &B, int s, uint32_t t) {
    const uint32_t W[8] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w};
    uint4 r;
    if (s == 0) {
        const uint32_t sel = t | ((2u + t) << 4) | ((4u + t) << 8) | ((6u + t) << 12);
        r.x = __byte_perm(W[0], W[1], sel); r.y = __byte_perm(W[2], W[3], sel);
        r.z = __byte_perm(W[4], W[5], sel); r.w = __byte_perm(W[6], W[7], sel);
    } else if (s == 1) {
        const uint32_t sel = (2u * t) | ((2u * t + 1u) << 4) | ((4u + 2u * t) << 8) | ((5u + 2u * t) << 12);
        r.x = __byte_perm(W[0], W[1], sel); r.y = __byte_perm(W[2], W[3], sel);
        r.z = __byte_perm(W[4], W[5], sel); r.w = __byte_perm(W[6], W[7], sel);
    } else if (s == 2) {
        r.x = t ? W[1] : W[0]; r.y = t ? W[3] : W[2]; r.z = t ? W[5] : W[4]; r.w = t ? W[7] : W[6];
    } else {
        r.x = t ? W[2] : W[0]; r.y = t ? W[3] : W[1]; r.z = t ? W[6] : W[4]; r.w = t ? W[7] : W[5];
    }
    return r;
}

}  // namespace tg
