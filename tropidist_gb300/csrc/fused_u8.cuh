// Register-resident update groups for uint8 tables (the inner loop of the fused tile pass).
//
// A group is a set of update ops of one pass whose chunk masks (mask >> 4: the part above the 16
// entries of a 16-byte chunk) span a subspace of dimension <= 3 of the tile's chunk index; the
// in-chunk part of a mask (bits 0..3) is free.  Let b0, b1, b2 be a reduced basis of that subspace
// extended to dimension 3, with pivot bits p0, p1, p2 (bit p_j set in b_j only).  The tile's chunks
// split into cosets {c0 ^ X[x] : x < 8}, X[x] = XOR of the b_j selected by the bits of x, c0
// ranging over the chunk indices with zero pivot bits.  Every update of the group pairs entries
// inside one coset, so a thread loads a whole coset (8 chunks = 128 entries) into registers,
// applies every update of the group there and writes it back: one shared-memory round trip per
// group.
//
// Register file: R[8x + 2k + p] holds entries 4k + p and 4k + p + 2 of chunk x as two 16-bit
// lanes (bytes p and p + 2 of word k), so min(a, b + w) is one __viaddmin_u16x2 for two entries
// (no wrap: entries and weights are below 256).  An update with chunk coordinates y (b-basis) and
// in-chunk mask m pairs register r with register r ^ X, X = 8y + 2(m >> 2) + (m & 1), and swaps
// the lanes of the partner when bit 1 of m is set; the code X | (lane swap) << 6 is dispatched
// through a switch to code unrolled by template recursion (every register index is a
// compile-time constant).
//
// Shared-memory tile slots are swizzled: chunk c lives in slot c ^ fold(c), fold(c) the XOR of
// the 3-bit groups of c above bit 2, so the 16-byte slots of 8 lanes that differ in three chunk
// bits of distinct residues mod 3 fall in distinct bank quads; the thread -> coset map of each
// group (tpos) puts such bits on the lanes of each quarter warp.
#pragma once
#include "tg_common.cuh"

namespace tg {

#define FP_MAXG 16

struct GroupDesc {
    uint32_t xoff[8];        // chunk offsets X[x] inside a coset
    uint8_t tpos[16];        // chunk bit receiving bit j of the coset number (non-pivot bits)
    uint8_t first, count;    // the group's codes: ucode[first .. first + count)
    uint8_t pad[2];
};

__device__ __forceinline__ uint32_t swap_halves(uint32_t v) { return __byte_perm(v, 0u, 0x1032); }

// shared-memory slot of tile chunk c (sm: 7 to swizzle, 0 for the plain layout)
__device__ __forceinline__ uint32_t tslot(uint32_t c, uint32_t sm) {
    return c ^ (((c >> 3) ^ (c >> 6) ^ (c >> 9) ^ (c >> 12) ^ (c >> 15)) & sm);
}

// a packed word (bytes e0..e3) as lanes (e0, e2) and (e1, e3), and back
__device__ __forceinline__ void unpack_eo(uint32_t w, uint32_t &e, uint32_t &o) {
    e = __byte_perm(w, 0u, 0x4240);
    o = __byte_perm(w, 0u, 0x4341);
}
__device__ __forceinline__ uint32_t pack_eo(uint32_t e, uint32_t o) { return __byte_perm(e, o, 0x6240); }

// register pairs (I, I ^ X) of one update, I ascending
template <int X, int HS, int I>
struct RegPairs {
    static __device__ __forceinline__ void run(uint32_t (&R)[64], uint32_t w2) {
        if constexpr (X == 0) {
            if constexpr (HS) R[I] = __viaddmin_u16x2(swap_halves(R[I]), w2, R[I]);
        } else if constexpr (I < (I ^ X)) {
            const uint32_t a = R[I], b = R[I ^ X];
            if constexpr (HS) {
                R[I] = __viaddmin_u16x2(swap_halves(b), w2, a);
                R[I ^ X] = __viaddmin_u16x2(swap_halves(a), w2, b);
            } else {
                R[I] = __viaddmin_u16x2(b, w2, a);
                R[I ^ X] = __viaddmin_u16x2(a, w2, b);
            }
        }
        if constexpr (I < 63) RegPairs<X, HS, I + 1>::run(R, w2);
    }
};

#define TG_RC(c) case c: RegPairs<((c) & 63), ((c) >> 6), 0>::run(R, w2); break;
#define TG_RC4(c) TG_RC(c) TG_RC(c + 1) TG_RC(c + 2) TG_RC(c + 3)
#define TG_RC16(c) TG_RC4(c) TG_RC4(c + 4) TG_RC4(c + 8) TG_RC4(c + 12)

// code: register xor (bits 0..5) | lane swap << 6
__device__ __forceinline__ void reg_dispatch(uint32_t code, uint32_t (&R)[64], uint32_t w2) {
    switch (code) {
        TG_RC16(0) TG_RC16(16) TG_RC16(32) TG_RC16(48) TG_RC16(64) TG_RC16(80) TG_RC16(96) TG_RC16(112)
        default: break;
    }
}

#undef TG_RC16
#undef TG_RC4
#undef TG_RC

// one group over a shared-memory tile of 2^d entries (chunks of 16 entries, swizzled slots),
// all threads of the block
template <int NT>
__device__ __forceinline__ void run_group(uint4 *TC, int d, const GroupDesc &g, const uint8_t *ucode,
                                          const uint8_t *uw) {
    const int nt = d - 4 - 3;
    const uint32_t ncos = 1u << nt;
    for (uint32_t k = threadIdx.x; k < ncos; k += NT) {
        uint32_t c0 = 0;
        for (int j = 0; j < nt; j++) c0 |= ((k >> j) & 1u) << g.tpos[j];
        uint32_t R[64];
#pragma unroll
        for (int x = 0; x < 8; x++) {
            const uint4 v = TC[tslot(c0 ^ g.xoff[x], 7u)];
            unpack_eo(v.x, R[8 * x + 0], R[8 * x + 1]);
            unpack_eo(v.y, R[8 * x + 2], R[8 * x + 3]);
            unpack_eo(v.z, R[8 * x + 4], R[8 * x + 5]);
            unpack_eo(v.w, R[8 * x + 6], R[8 * x + 7]);
        }
        for (int u = 0; u < g.count; u++) {
            const uint32_t w = uw[g.first + u];
            reg_dispatch(ucode[g.first + u], R, w | (w << 16));
        }
#pragma unroll
        for (int x = 0; x < 8; x++)
            TC[tslot(c0 ^ g.xoff[x], 7u)] = make_uint4(pack_eo(R[8 * x], R[8 * x + 1]), pack_eo(R[8 * x + 2], R[8 * x + 3]),
                                                      pack_eo(R[8 * x + 4], R[8 * x + 5]), pack_eo(R[8 * x + 6], R[8 * x + 7]));
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
