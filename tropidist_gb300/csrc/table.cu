// Completion tables of the weight-bounded search on the GPU (cdist/gmitm.c:36-186).
//
// A table maps the syndrome hash of every column subset of size <= k to its least size.  Slot
// index = zh & (slots - 1); keys as the reference: compact tables store key = (zl & 0x7FFF...0000)
// | (label & 0xFFFF) | 1 << 63 in one 64-bit word (cdist/gmitm.c:46-48), wide tables (more than 16
// observables) store the 63-bit fingerprint zl | 1 << 63 and the full label in a 16-byte slot
// claimed with one 128-bit compare-and-swap.  Costs are one byte per slot (255 = empty).
//
// Build: one thread per subset, the subsets of size s unranked in the combinatorial number system
// from a binomial table, one launch per size s = 0..k in increasing order; the thread that creates a
// key writes its cost, and since every later launch has a larger size, the first cost of a key is
// its minimum: no atomic min on the cost byte is needed.
// Lookup (cdist/gmitm.c:138-163): least cost <= R among the entries with the probe's fingerprint and
// a label different from the probe's, scanning from the slot until an empty slot.
#include "tg_common.cuh"
#include "tg_capi.h"

#include <cstring>
#include <vector>

namespace tg {

#define TB_FPMASK 0x7FFFFFFFFFFF0000ull
#define TB_MAXK 8

struct TableHandle {
    int log2slots;
    int wide;
    uint64_t slots;
    unsigned long long *keys;      // compact: keys[slots]; wide: pairs (key, label) [2 * slots]
    uint8_t *cost;                 // [slots]
    unsigned long long *count;     // device counter of entries
    int64_t entries;
    int k;
    size_t keys_bytes, cost_bytes;  // allocated sizes (a reused buffer may be larger)
};

__device__ __forceinline__ uint64_t tb_compact_key(uint64_t zl, uint64_t lg) {
    return (zl & TB_FPMASK) | (lg & 0xFFFFull) | (1ull << 63);
}

// subset of size s with colex rank r: c_s > ... > c_1, C(c_j, j) <= remaining rank
__device__ __forceinline__ void tb_unrank(uint64_t r, int s, int n, const unsigned long long *binom, int *cols) {
    int hi = n;   // exclusive bound for c_s
    for (int j = s; j >= 1; j--) {
        // largest c in [j-1, hi) with C(c, j) <= r
        int lo = j - 1, top = hi - 1;
        while (lo < top) {
            int mid = (lo + top + 1) >> 1;
            if (binom[(uint64_t)mid * (TB_MAXK + 1) + j] <= r) lo = mid;
            else top = mid - 1;
        }
        cols[j - 1] = lo;
        r -= binom[(uint64_t)lo * (TB_MAXK + 1) + j];
        hi = lo;
    }
}

__global__ void k_tb_clear(unsigned long long *keys, uint64_t nwords, uint8_t *cost, uint64_t slots) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nwords; i += stride) keys[i] = 0ull;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < slots; i += stride) cost[i] = 255;
}

__global__ void k_tb_build(TableHandle T, int s, uint64_t nsub, int n, const unsigned long long *binom,
                           const unsigned long long *zh, const unsigned long long *zl, const unsigned long long *lg,
                           unsigned long long *errflag) {
    const uint64_t mask = T.slots - 1;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < nsub; r += (uint64_t)gridDim.x * blockDim.x) {
        int cols[TB_MAXK];
        tb_unrank(r, s, n, binom, cols);
        uint64_t h = 0, l = 0, g = 0;
        for (int j = 0; j < s; j++) { h ^= zh[cols[j]]; l ^= zl[cols[j]]; g ^= lg[cols[j]]; }
        uint64_t i = h & mask;
        bool done = false;
        if (!T.wide) {
            const uint64_t key = tb_compact_key(l, g);
            for (uint64_t probe = 0; probe <= mask && !done; probe++) {
                unsigned long long cur = T.keys[i];
                if (cur == 0ull) {
                    unsigned long long prev = atomicCAS(T.keys + i, 0ull, (unsigned long long)key);
                    if (prev == 0ull) {
                        T.cost[i] = (uint8_t)s;
                        agg_inc(T.count);
                        done = true;
                        break;
                    }
                    cur = prev;
                }
                if (cur == key) { done = true; break; }
                i = (i + 1) & mask;
            }
        } else {
            const uint64_t key = l | (1ull << 63);
            for (uint64_t probe = 0; probe <= mask && !done; probe++) {
                unsigned __int128 *slot = reinterpret_cast<unsigned __int128 *>(T.keys) + i;
                unsigned __int128 cur = *slot;
                const unsigned __int128 want = ((unsigned __int128)g << 64) | key;
                if (cur == 0) {
                    unsigned __int128 prev = atomicCAS(slot, (unsigned __int128)0, want);
                    if (prev == 0) {
                        T.cost[i] = (uint8_t)s;
                        agg_inc(T.count);
                        done = true;
                        break;
                    }
                    cur = prev;
                }
                if (cur == want) { done = true; break; }
                i = (i + 1) & mask;
            }
        }
        if (!done) atomicOr(errflag, 1ull);
    }
}

__global__ void k_tb_lookup(TableHandle T, uint64_t m, const unsigned long long *zh, const unsigned long long *zl,
                            const unsigned long long *lg, const int *R, int *out) {
    const uint64_t mask = T.slots - 1;
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < m; q += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t i = zh[q] & mask;
        int best = -1;
        const int rq = R[q];
        if (!T.wide) {
            const uint64_t fp = zl[q] & TB_FPMASK, lab = lg[q] & 0xFFFFull;
            for (uint64_t probe = 0; probe <= mask; probe++) {
                const unsigned long long cur = T.keys[i];
                if (cur == 0ull) break;
                if ((cur & TB_FPMASK) == fp && (cur & 0xFFFFull) != lab) {
                    const int c = T.cost[i];
                    if (c <= rq && (best < 0 || c < best)) best = c;
                }
                i = (i + 1) & mask;
            }
        } else {
            const uint64_t key = zl[q] | (1ull << 63);
            for (uint64_t probe = 0; probe <= mask; probe++) {
                const unsigned long long ck = T.keys[2 * i], cl = T.keys[2 * i + 1];
                if (ck == 0ull && cl == 0ull) break;
                if (ck == key && cl != lg[q]) {
                    const int c = T.cost[i];
                    if (c <= rq && (best < 0 || c < best)) best = c;
                }
                i = (i + 1) & mask;
            }
        }
        out[q] = best;
    }
}

// One released allocation of each kind per host thread, handed to the next request that fits: a
// search creates and frees a table and its probe buffers per call, and cudaMalloc, cudaMallocHost,
// cudaFreeHost and the device-synchronizing cudaFree cost tens to hundreds of microseconds each.
struct Reuse {
    void *p = nullptr;
    size_t bytes = 0;
};
enum { RU_KEYS, RU_COST, RU_COUNT, RU_BUILD, RU_DIN, RU_DOUT, RU_HIN, RU_HOUT, RU_N };
static thread_local Reuse g_reuse[RU_N];

static bool ru_host(int kind) { return kind == RU_HIN || kind == RU_HOUT; }

static void ru_release(int kind, void *p) {
    if (ru_host(kind)) cudaFreeHost(p);
    else cudaFree(p);
}

// a buffer of at least `bytes` (*got: its size), from the cache or newly allocated; null on failure
static void *ru_take(int kind, size_t bytes, size_t *got) {
    Reuse &r = g_reuse[kind];
    if (r.p && r.bytes >= bytes) {
        void *p = r.p;
        *got = r.bytes;
        r.p = nullptr;
        r.bytes = 0;
        return p;
    }
    void *p = nullptr;
    const cudaError_t e = ru_host(kind) ? cudaMallocHost(&p, bytes) : cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    *got = bytes;
    return p;
}

// back to the cache (the larger of the two buffers stays)
static void ru_give(int kind, void *p, size_t bytes) {
    if (!p) return;
    Reuse &r = g_reuse[kind];
    if (r.p && r.bytes >= bytes) {
        ru_release(kind, p);
        return;
    }
    if (r.p) ru_release(kind, r.p);
    r.p = p;
    r.bytes = bytes;
}

static unsigned tb_grid(uint64_t items) {
    uint64_t g = (items + 255) / 256;
    uint64_t cap = (uint64_t)sm_count() * 16;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace tg

using namespace tg;

extern "C" {

// cdist/gmitm.c:61-76 tab_create: a table of 2^log2slots slots (wide: full labels).  NULL (and
// *status = -3) when the device memory cannot be allocated.
void *tg_tab_create(int log2slots, int wide, int *status) {
    int st = TG_OK;
    TableHandle *T = nullptr;
    if (log2slots < 1 || log2slots > 40) st = set_error(TG_ERR_ARG, "log2slots out of range");
    else {
        T = new TableHandle();
        memset(T, 0, sizeof(*T));
        T->log2slots = log2slots;
        T->wide = wide ? 1 : 0;
        T->slots = 1ull << log2slots;
        const uint64_t nwords = T->slots * (wide ? 2 : 1);
        size_t cb = 0;
        T->keys = static_cast<unsigned long long *>(ru_take(RU_KEYS, nwords * 8, &T->keys_bytes));
        T->cost = static_cast<uint8_t *>(ru_take(RU_COST, T->slots, &T->cost_bytes));
        T->count = static_cast<unsigned long long *>(ru_take(RU_COUNT, 8, &cb));
        if (!T->keys || !T->cost || !T->count) {
            ru_give(RU_KEYS, T->keys, T->keys_bytes);
            ru_give(RU_COST, T->cost, T->cost_bytes);
            ru_give(RU_COUNT, T->count, 8);
            delete T;
            T = nullptr;
            st = set_error(TG_ERR_NOMEM, "device table allocation failed");
        } else {
            // cleared before the call returns: lookups may come on any stream
            k_tb_clear<<<tb_grid(nwords), 256>>>(T->keys, nwords, T->cost, T->slots);
            st = cuda_check(cudaMemsetAsync(T->count, 0, 8, 0), "table clear");
            if (!st) st = cuda_check(cudaStreamSynchronize(0), "table clear");
        }
    }
    if (status) *status = st;
    return T;
}

void tg_tab_free(void *p) {
    TableHandle *T = static_cast<TableHandle *>(p);
    if (!T) return;
    cudaDeviceSynchronize();        // kernels still reading the table finish before it is reused
    ru_give(RU_KEYS, T->keys, T->keys_bytes);
    ru_give(RU_COST, T->cost, T->cost_bytes);
    ru_give(RU_COUNT, T->count, 8);
    delete T;
}

int64_t tg_tab_count(void *p) { return p ? static_cast<TableHandle *>(p)->entries : -1; }

int64_t tg_tab_slots_log2(void *p) { return p ? static_cast<TableHandle *>(p)->log2slots : -1; }

// cdist/gmitm.c:176-186 tab_build: every subset of size 0..k of the n columns (hashes zh, zl and
// labels lg are HOST arrays of n uint64).
int tg_tab_build(void *p, int n, const uint64_t *zh, const uint64_t *zl, const uint64_t *lg, int k) {
    TableHandle *T = static_cast<TableHandle *>(p);
    if (!T || n < 0 || k < 0 || (n > 0 && (!zh || !zl || !lg))) return set_error(TG_ERR_ARG, "bad table build");
    if (k > TB_MAXK) return set_error(TG_ERR_TOO_BIG, "table depth beyond 8");
    k = std::min(k, n);
    T->k = k;
    // binomials C(c, j) for c <= n, j <= k
    std::vector<unsigned long long> binom((uint64_t)(n + 1) * (TB_MAXK + 1), 0ull);
    for (int c = 0; c <= n; c++) {
        binom[(uint64_t)c * (TB_MAXK + 1)] = 1;
        for (int j = 1; j <= TB_MAXK && j <= c; j++)
            binom[(uint64_t)c * (TB_MAXK + 1) + j] = binom[(uint64_t)(c - 1) * (TB_MAXK + 1) + j - 1] +
                                                     (j <= c - 1 ? binom[(uint64_t)(c - 1) * (TB_MAXK + 1) + j] : 0ull);
    }
    const size_t nb = binom.size() * 8, nh = (size_t)std::max(n, 1) * 8, tot = nb + 3 * nh + 8;
    size_t dbytes = 0, hbytes = 0;
    unsigned long long *d = static_cast<unsigned long long *>(ru_take(RU_BUILD, tot, &dbytes));
    if (!d) return set_error(TG_ERR_NOMEM, "device buffers for the build");
    // the binomials, hashes and labels staged in pinned memory and sent in one copy; the error
    // flag and the entry count come back in one copy (one synchronization for the whole build)
    uint8_t *h = static_cast<uint8_t *>(ru_take(RU_HIN, tot, &hbytes));
    if (!h) {
        ru_give(RU_BUILD, d, dbytes);
        return set_error(TG_ERR_NOMEM, "pinned staging for the build");
    }
    memcpy(h, binom.data(), nb);
    if (n) {
        memcpy(h + nb, zh, (size_t)n * 8);
        memcpy(h + nb + nh, zl, (size_t)n * 8);
        memcpy(h + nb + 2 * nh, lg, (size_t)n * 8);
    }
    memset(h + nb + 3 * nh, 0, 8);
    unsigned long long *dbin = d, *dzh = d + binom.size(), *dzl = dzh + std::max(n, 1), *dlg = dzl + std::max(n, 1);
    unsigned long long *derr = dlg + std::max(n, 1);
    cudaStream_t st = 0;
    int e = cuda_check(cudaMemcpyAsync(d, h, tot, cudaMemcpyHostToDevice, st), "build inputs");
    for (int s = 0; s <= k && !e; s++) {
        const uint64_t nsub = binom[(uint64_t)n * (TB_MAXK + 1) + s];
        k_tb_build<<<tb_grid(nsub), 256, 0, st>>>(*T, s, nsub, n, dbin, dzh, dzl, dlg, derr);
        e = cuda_check(cudaGetLastError(), "table build");
    }
    unsigned long long *hr = reinterpret_cast<unsigned long long *>(h);
    if (!e) e = cuda_check(cudaMemcpyAsync(hr, derr, 8, cudaMemcpyDeviceToHost, st), "flag read");
    if (!e) e = cuda_check(cudaMemcpyAsync(hr + 1, T->count, 8, cudaMemcpyDeviceToHost, st), "count read");
    if (!e) e = cuda_check(cudaStreamSynchronize(st), "build sync");
    const unsigned long long err = e ? 0 : hr[0], cnt = e ? 0 : hr[1];
    ru_give(RU_HIN, h, hbytes);
    ru_give(RU_BUILD, d, dbytes);
    if (e) return e;
    if (err) return set_error(TG_ERR_TOO_BIG, "completion table full");
    T->entries = (int64_t)cnt;
    return TG_OK;
}

// Batched probes (DEVICE arrays of m entries): out[q] = least cost <= R[q] among the entries with
// the fingerprint of (zh[q], zl[q]) and a label other than lg[q], or -1.
int tg_tab_lookup_dev(void *p, uint64_t m, const void *zh, const void *zl, const void *lg, const void *R, void *out,
                      void *stream) {
    TableHandle *T = static_cast<TableHandle *>(p);
    if (!T || (m && (!zh || !zl || !lg || !R || !out))) return set_error(TG_ERR_ARG, "bad lookup");
    if (m) k_tb_lookup<<<tb_grid(m), 256, 0, (cudaStream_t)stream>>>(*T, m, (const unsigned long long *)zh,
                                                                      (const unsigned long long *)zl,
                                                                      (const unsigned long long *)lg, (const int *)R,
                                                                      (int *)out);
    return cuda_check(cudaGetLastError(), "table lookup");
}

// A native answer to the search's probe waves (tg_probe_fn): a wave's probes go through pinned
// staging to the device table and back on a stream of its own, with no interpreter in the loop.
struct NativeProbe {
    TableHandle *T;
    int64_t cap;                   // probes per round trip
    uint8_t *h_in, *d_in;          // zh, zl, lg (8 bytes each) and R (4 bytes): 28 bytes per probe
    int32_t *h_out, *d_out;
    size_t b_hin, b_din, b_hout, b_dout;
    cudaStream_t st;
};

static thread_local cudaStream_t g_probe_stream = nullptr;    // one probe stream per host thread, kept

static void probe_release(NativeProbe *P) {
    if (!P) return;
    if (P->st) cudaStreamSynchronize(P->st);
    ru_give(RU_HIN, P->h_in, P->b_hin);
    ru_give(RU_HOUT, P->h_out, P->b_hout);
    ru_give(RU_DIN, P->d_in, P->b_din);
    ru_give(RU_DOUT, P->d_out, P->b_dout);
    delete P;
}

// The reference's own names and signatures (cdist/search.py:58-67 binds them with ctypes), so a
// binding written for cdist's libgmitm can load this library unchanged: NULL from tab_create when
// the table cannot be allocated (the reference's binding raises MemoryError on NULL), tab_build on
// HOST arrays zh, zl, lg of n columns.
void *tg_tab_probe_create(void *table, int64_t cap, int *status) {
    int st = TG_OK;
    NativeProbe *P = nullptr;
    if (!table || cap < 1 || cap > (1ll << 28)) {
        st = set_error(TG_ERR_ARG, "bad table or probe capacity");
    } else {
        P = new NativeProbe();
        memset(P, 0, sizeof(*P));
        P->T = static_cast<TableHandle *>(table);
        P->cap = cap;
        P->h_in = static_cast<uint8_t *>(ru_take(RU_HIN, 28 * (size_t)cap, &P->b_hin));
        P->h_out = static_cast<int32_t *>(ru_take(RU_HOUT, 4 * (size_t)cap, &P->b_hout));
        P->d_in = static_cast<uint8_t *>(ru_take(RU_DIN, 28 * (size_t)cap, &P->b_din));
        P->d_out = static_cast<int32_t *>(ru_take(RU_DOUT, 4 * (size_t)cap, &P->b_dout));
        if (!g_probe_stream) st = cuda_check(cudaStreamCreateWithFlags(&g_probe_stream, cudaStreamNonBlocking),
                                             "probe stream");
        P->st = g_probe_stream;
        if (!st && (!P->h_in || !P->h_out || !P->d_in || !P->d_out)) st = set_error(TG_ERR_NOMEM, "probe buffers");
        if (st) {
            probe_release(P);
            P = nullptr;
            if (st == TG_ERR_CUDA) st = set_error(TG_ERR_NOMEM, "probe buffers");
        }
    }
    if (status) *status = st;
    return P;
}

int tg_tab_probe(int64_t m, const uint64_t *zh, const uint64_t *zl, const uint64_t *lg, const int32_t *R,
                 int32_t *out, void *ctx) {
    NativeProbe *P = static_cast<NativeProbe *>(ctx);
    if (!P || m < 0 || (m && (!zh || !zl || !lg || !R || !out))) return 1;
    for (int64_t off = 0; off < m; off += P->cap) {
        const int64_t n = m - off < P->cap ? m - off : P->cap;
        memcpy(P->h_in, zh + off, 8 * (size_t)n);
        memcpy(P->h_in + 8 * n, zl + off, 8 * (size_t)n);
        memcpy(P->h_in + 16 * n, lg + off, 8 * (size_t)n);
        memcpy(P->h_in + 24 * n, R + off, 4 * (size_t)n);
        if (cudaMemcpyAsync(P->d_in, P->h_in, 28 * (size_t)n, cudaMemcpyHostToDevice, P->st) != cudaSuccess) return 1;
        k_tb_lookup<<<tb_grid(n), 256, 0, P->st>>>(*P->T, n, (const unsigned long long *)P->d_in,
                                                   (const unsigned long long *)(P->d_in + 8 * n),
                                                   (const unsigned long long *)(P->d_in + 16 * n),
                                                   (const int *)(P->d_in + 24 * n), P->d_out);
        if (cudaGetLastError() != cudaSuccess) return 1;
        if (cudaMemcpyAsync(P->h_out, P->d_out, 4 * (size_t)n, cudaMemcpyDeviceToHost, P->st) != cudaSuccess) return 1;
        if (cudaStreamSynchronize(P->st) != cudaSuccess) return 1;
        memcpy(out + off, P->h_out, 4 * (size_t)n);
    }
    return 0;
}

void tg_tab_probe_free(void *ctx) { probe_release(static_cast<NativeProbe *>(ctx)); }

void *tab_create(int log2slots, int wide) {
    int status = 0;
    return tg_tab_create(log2slots, wide, &status);
}

void tab_free(void *t) { tg_tab_free(t); }

int64_t tab_count(void *t) { return tg_tab_count(t); }

void tab_build(void *t, int n, const uint64_t *zh, const uint64_t *zl, const uint64_t *lg, int k) {
    tg_tab_build(t, n, zh, zl, lg, k);
}

}  // extern "C"
