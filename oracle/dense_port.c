/* C/OpenMP port of the reference's dense Rank DP kernels: TEST INFRASTRUCTURE ONLY (the timed
 * CPU baseline and a fast checker for large tables).  Portable C (no vector intrinsics), so it
 * builds the same on x86-64 and aarch64.
 *
 *   port_update          cdist/viterbi.c:73-118   T[s] = min(T[s], sat(T[s^h] + 1)), 64-entry blocks
 *   port_expand_update   cdist/viterbi.c:122-138  U[s ^ hl] = sat(T[s] + 1) into the upper half
 *   port_select          cdist/viterbi.c:155-172  keep bit pos == target, drop the bit (in place)
 *   port_fill            cdist/viterbi.c:174-179
 *   port_hist            cdist/viterbi.c:182-193
 *   port_run_plan        cdist/kernel.py:94-138   the executor loop (expand fused with the update of
 *                                                 the starting column, as the reference does)
 * Op stream: int64 triples (code, a, b): 0 expand, 1 update(mask, w), 2 select(pos, target).
 */
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define INF8 255

static inline uint8_t sat1(uint8_t v) { return (uint8_t)(v + (v != INF8)); }
static inline uint8_t satw(uint8_t v, int w) {
    unsigned x = (unsigned)v + (unsigned)w;
    return (uint8_t)(v == INF8 || x > INF8 ? INF8 : x);
}

/* pairs (x[i], y[i ^ m]) for i < 64 */
static inline void pair_block(uint8_t *x, uint8_t *y, unsigned m) {
    if (m == 0) {
        for (int i = 0; i < 64; i++) {
            uint8_t a = x[i], b = y[i];
            uint8_t a1 = sat1(a), b1 = sat1(b);
            x[i] = a < b1 ? a : b1;
            y[i] = b < a1 ? b : a1;
        }
    } else {
        for (int i = 0; i < 64; i++) {
            uint8_t a = x[i ^ m], b = y[i];
            uint8_t a1 = sat1(a), b1 = sat1(b);
            x[i ^ m] = a < b1 ? a : b1;
            y[i] = b < a1 ? b : a1;
        }
    }
}

void port_update(uint8_t *T, uint64_t n, uint64_t h) {
    if (h == 0 || n < 2) return;
    int hb = 63 - __builtin_clzll(h);
    uint64_t half = 1ULL << hb, hl = h ^ half;
    if (n >= 128 && hb >= 6) {
        uint64_t hi = hl & ~63ULL, nblk = n >> 6, hbb = half >> 6;
        unsigned m = (unsigned)(hl & 63);
        #pragma omp parallel for schedule(static)
        for (uint64_t b = 0; b < nblk; b++) {
            if (b & hbb) continue;
            pair_block(T + (b << 6), T + ((((b << 6) ^ hi)) | half), m);
        }
    } else if (n >= 128) {
        uint64_t nblk = n >> 6;
        #pragma omp parallel for schedule(static)
        for (uint64_t b = 0; b < nblk; b++) {
            uint8_t *B = T + (b << 6);
            for (unsigned s = 0; s < 64; s++) {
                if (s & half) continue;
                unsigned t = s ^ (unsigned)h;
                uint8_t a = B[s], c = B[t];
                uint8_t a1 = sat1(a), c1 = sat1(c);
                B[s] = a < c1 ? a : c1;
                B[t] = c < a1 ? c : a1;
            }
        }
    } else {
        for (uint64_t s = 0; s < n; s++) {
            if (s & half) continue;
            uint64_t t = s ^ h;
            uint8_t a = T[s], c = T[t];
            uint8_t a1 = sat1(a), c1 = sat1(c);
            T[s] = a < c1 ? a : c1;
            T[t] = c < a1 ? c : a1;
        }
    }
}

void port_update_w(uint8_t *T, uint64_t n, uint64_t h, int w) {
    if (h == 0 || n < 2) return;
    int hb = 63 - __builtin_clzll(h);
    uint64_t half = 1ULL << hb;
    #pragma omp parallel for schedule(static) if (n >= (1ULL << 16))
    for (uint64_t s = 0; s < n; s++) {
        if (s & half) continue;
        uint64_t t = s ^ h;
        uint8_t a = T[s], c = T[t];
        uint8_t aw = satw(a, w), cw = satw(c, w);
        T[s] = a < cw ? a : cw;
        T[t] = c < aw ? c : aw;
    }
}

void port_expand_update(uint8_t *T, uint64_t n, uint64_t hl) {
    uint8_t *U = T + n;
    if (n >= 64) {
        uint64_t hi = hl & ~63ULL, nblk = n >> 6;
        unsigned m = (unsigned)(hl & 63);
        #pragma omp parallel for schedule(static)
        for (uint64_t b = 0; b < nblk; b++) {
            const uint8_t *x = T + (b << 6);
            uint8_t *y = U + ((b << 6) ^ hi);
            for (int i = 0; i < 64; i++) y[i ^ m] = sat1(x[i]);
        }
    } else {
        for (uint64_t s = 0; s < n; s++) U[s ^ hl] = sat1(T[s]);
    }
}

static void copy_par(uint8_t *dst, const uint8_t *src, uint64_t len) {
    const uint64_t chunk = 1ULL << 20;
    if (len <= 4 * chunk) { memmove(dst, src, len); return; }
    #pragma omp parallel for schedule(static)
    for (uint64_t o = 0; o < len; o += chunk)
        memcpy(dst + o, src + o, (len - o < chunk) ? (len - o) : chunk);
}

uint64_t port_select(uint8_t *T, uint64_t n, int pos, int target) {
    uint64_t blk = 1ULL << pos, nb = n >> (pos + 1);
    if (nb == 0) return n;
    if (target) copy_par(T, T + blk, blk);
    if (blk >= (1ULL << 22)) {
        for (uint64_t k = 1; k < nb; k++) copy_par(T + k * blk, T + (2 * k + (uint64_t)target) * blk, blk);
    } else {
        /* output block k reads input block 2k+target: for k in [a, 2a) every write lies below
           block 2a and every read at or above it */
        for (uint64_t a = 1; a < nb; a <<= 1) {
            uint64_t hi = (2 * a < nb) ? 2 * a : nb;
            #pragma omp parallel for schedule(static) if (hi - a > 64)
            for (uint64_t k = a; k < hi; k++) memcpy(T + k * blk, T + (2 * k + (uint64_t)target) * blk, blk);
        }
    }
    return n >> 1;
}

void port_fill(uint8_t *T, uint64_t n, uint8_t v) {
    const uint64_t chunk = 1ULL << 22;
    if (n <= chunk) { memset(T, v, n); return; }
    #pragma omp parallel for schedule(static)
    for (uint64_t o = 0; o < n; o += chunk) memset(T + o, v, (n - o < chunk) ? (n - o) : chunk);
}

void port_hist(const uint8_t *T, uint64_t n, uint64_t *hist) {
    for (int v = 0; v < 256; v++) hist[v] = 0;
    #pragma omp parallel
    {
        uint64_t loc[256];
        for (int v = 0; v < 256; v++) loc[v] = 0;
        #pragma omp for schedule(static) nowait
        for (uint64_t s = 0; s < n; s++) loc[T[s]]++;
        #pragma omp critical
        for (int v = 0; v < 256; v++) hist[v] += loc[v];
    }
}

int port_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* Threads of the following parallel regions (the 1-thread leg of the CPU baseline). */
void port_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* Runs ops[0..nops) on buf (room for the largest table); returns the final table size.  The
   first entry of buf must be initialised by the caller (0 for a fresh sweep). */
uint64_t port_run_plan(const int64_t *ops, int64_t nops, uint8_t *buf, uint64_t n) {
    int64_t i = 0;
    while (i < nops) {
        int64_t code = ops[3 * i], a = ops[3 * i + 1], b = ops[3 * i + 2];
        if (code == 0) {
            int bits = 63 - __builtin_clzll(n);
            if (i + 1 < nops && ops[3 * (i + 1)] == 1 && ops[3 * (i + 1) + 2] == 1 &&
                ((uint64_t)ops[3 * (i + 1) + 1] >> bits) == 1) {
                port_expand_update(buf, n, (uint64_t)ops[3 * (i + 1) + 1] ^ n);
                n <<= 1;
                i += 2;
                continue;
            }
            port_fill(buf + n, n, INF8);
            n <<= 1;
        } else if (code == 1) {
            if (b == 1) port_update(buf, n, (uint64_t)a);
            else port_update_w(buf, n, (uint64_t)a, (int)b);
        } else {
            n = port_select(buf, n, (int)a, (int)b);
        }
        i++;
    }
    return n;
}
