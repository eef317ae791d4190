/* C port of the reference's tree DP join (cdist/tree_dp.c:13-39): TEST INFRASTRUCTURE ONLY, the
 * timed CPU baseline of the tree DP.  The pairs i in [start, stop) of a join are visited in Gray
 * order: pair i has state XOR of the maps of the set bits of gray(i) = i ^ (i >> 1), and moving
 * from i to i + 1 toggles generator ctz(i + 1).  Single-threaded, no allocation, like the
 * reference's kernel. */
#include <stdint.h>

#define PORT_JOIN(T, NAME)                                                                        \
void NAME(const T *left, const T *right, T *out, const uint64_t *lm, const uint64_t *rm,           \
          unsigned parent_bits, uint64_t start, uint64_t stop, uint64_t inf) {                     \
    uint64_t l = 0, r = 0, p = 0;                                                                  \
    const uint64_t pmask = parent_bits >= 64 ? ~0ull : ((1ull << parent_bits) - 1ull);            \
    for (uint64_t g = start ^ (start >> 1), b = 0; g; g >>= 1, b++)                                \
        if (g & 1) { l ^= lm[b]; r ^= rm[b]; p ^= (1ull << b) & pmask; }                          \
    for (uint64_t i = start; i < stop; i++) {                                                      \
        const uint64_t a = left[l], c = right[r];                                                  \
        if (a < inf && c < inf && a + c <= inf && a + c < out[p]) out[p] = (T)(a + c);             \
        const uint64_t nx = i + 1;                                                                 \
        if (nx < stop) {                                                                           \
            const unsigned k = (unsigned)__builtin_ctzll(nx);                                      \
            l ^= lm[k]; r ^= rm[k];                                                                \
            if (k < parent_bits) p ^= 1ull << k;                                                   \
        }                                                                                          \
    }                                                                                              \
}

PORT_JOIN(uint8_t, tree_join_port_u8)
PORT_JOIN(uint16_t, tree_join_port_u16)
PORT_JOIN(uint32_t, tree_join_port_u32)
