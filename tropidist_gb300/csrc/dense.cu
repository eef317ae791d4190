// Dense Rank DP on the GPU: per-op kernels (the reference's C-ABI on device buffers), the
// single-CTA shared-memory sweep for narrow tables, the fused multi-column tile pass for wide
// tables, and the host scheduler that turns a plan's op stream into launches.
//
// Table layout in HBM: entry s of a width-w table at index s (uint8 or uint16), bit p of s = the
// partial parity of the p-th active row (rows in order of activation), exactly as in
// cdist/kernel.py:94-138.  Tables are ping-ponged between two caller-owned buffers.
//
// Fused pass.  Update ops commute (each is a min-plus convolution over (Z_2)^w), an update
// commutes with the expand / select of a row it does not touch, an expand can be replaced by
// "the new row's bit-1 half starts at INF", and a select can be deferred to the store.  So a run
// of consecutive ops is one pass over the table as long as the rows it touches, plus the rows at
// the lowest 4 input and output positions (16-byte contiguity), number at most DMAX: the table is
// cut into tiles of 2^d entries that vary exactly in those rows, each tile is loaded into shared
// memory, every update of the run is applied there, and the entries on the selected halves are
// stored to their positions in the output layout.
#include "tg_common.cuh"
#include "tg_capi.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace tg {

// ------------------------------------------------------------------ library state
thread_local std::string g_err;
static int g_sm_count = 0;
static cudaStream_t g_stream = 0;

int set_error(int code, const char *what) {
    g_err = what;
    return code;
}
int cuda_check(cudaError_t e, const char *where) {
    if (e == cudaSuccess) return TG_OK;
    g_err = std::string(where) + ": " + cudaGetErrorString(e);
    return TG_ERR_CUDA;
}
int sm_count() {
    if (g_sm_count == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
        if (g_sm_count <= 0) g_sm_count = 1;
    }
    return g_sm_count;
}
cudaStream_t cur_stream() { return g_stream; }

// ------------------------------------------------------------------ per-op kernels (global memory)
// T[s] = min(T[s], T[s ^ h] + w) over a 2^bits table, 16-byte chunks, in place (pairs are disjoint)
template <typename E>
__global__ void k_update_chunks(E *__restrict__ T, int bits, uint64_t h, uint32_t w) {
    constexpr int CB = Entry<E>::CB;
    const uint64_t hhi = h >> CB;
    const uint32_t hlo = (uint32_t)(h & ((1u << CB) - 1));
    const uint64_t nch = 1ull << (bits - CB);
    Chunk *C = reinterpret_cast<Chunk *>(T);
    if (hhi == 0) {
        for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < nch; c += (uint64_t)gridDim.x * blockDim.x) {
            Chunk a = ld_chunk(C + c);
            st_chunk(C + c, chunk_minplus<E>(a, chunk_xor<E>(a, hlo), w));
        }
        return;
    }
    const int hb = 63 - __clzll(hhi);
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < nch / 2; p += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t c = insert_zero64(p, hb), c2 = c ^ hhi;
        Chunk a = ld_chunk(C + c), pb = chunk_xor<E>(ld_chunk(C + c2), hlo);
        chunk_minplus_pair<E>(a, pb, w);
        st_chunk(C + c, a);
        st_chunk(C + c2, chunk_xor<E>(pb, hlo));
    }
}

template <typename E>
__global__ void k_update_scalar(E *T, uint64_t n, uint64_t h, uint32_t w) {
    const int hb = 63 - __clzll(h);
    for (uint64_t p = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; p < n / 2; p += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t s = insert_zero64(p, hb), t = s ^ h;
        E a = T[s], b = T[t];
        T[s] = minplus1<E>(a, b, w);
        T[t] = minplus1<E>(b, a, w);
    }
}

// U[s ^ hl] = sat(T[s] + 1) with U = T + n (the new top row is flipped by the starting column)
template <typename E>
__global__ void k_expand_update(E *__restrict__ T, int bits, uint64_t hl, uint32_t w) {
    constexpr int CB = Entry<E>::CB;
    const uint64_t n = 1ull << bits;
    E *U = T + n;
    if (bits >= CB) {
        const uint64_t nch = n >> CB, hhi = hl >> CB;
        const uint32_t hlo = (uint32_t)(hl & ((1u << CB) - 1));
        const Chunk *A = reinterpret_cast<const Chunk *>(T);
        Chunk *B = reinterpret_cast<Chunk *>(U);
        Chunk inf;
        inf.w[0] = inf.w[1] = inf.w[2] = inf.w[3] = 0xFFFFFFFFu;
        for (uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; c < nch; c += (uint64_t)gridDim.x * blockDim.x) {
            Chunk a = chunk_xor<E>(ld_chunk(A + c), hlo);
            st_chunk(B + (c ^ hhi), chunk_minplus<E>(inf, a, w));
        }
    } else {
        for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x)
            U[s ^ hl] = minplus1<E>((E)Entry<E>::INF, T[s], w);
    }
}

__device__ unsigned long long g_hist_dev[256];

__global__ void k_hist(const uint8_t *__restrict__ T, uint64_t n, unsigned long long *hist) {
    __shared__ unsigned int loc[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) loc[i] = 0;
    __syncthreads();
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < n; s += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&loc[T[s]], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        if (loc[i]) atomicAdd(hist + i, (unsigned long long)loc[i]);
}

static unsigned grid_for(uint64_t items, int threads) {
    uint64_t g = (items + threads - 1) / threads;
    uint64_t cap = (uint64_t)sm_count() * 8;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (unsigned)g;
}

template <typename E>
int launch_update(E *T, uint64_t n, uint64_t h, uint32_t w, cudaStream_t st) {
    if (h == 0 || n < 2) return TG_OK;
    if (n & (n - 1)) return set_error(TG_ERR_ARG, "table size must be a power of two");
    if (h >= n) return set_error(TG_ERR_ARG, "update mask has bits beyond the table");
    const int bits = 63 - __builtin_clzll(n);
    if (bits >= Entry<E>::CB + 1 || (bits >= Entry<E>::CB && (h >> Entry<E>::CB) == 0)) {
        uint64_t items = (h >> Entry<E>::CB) ? (n >> (Entry<E>::CB + 1)) : (n >> Entry<E>::CB);
        k_update_chunks<E><<<grid_for(items, 256), 256, 0, st>>>(T, bits, h, w);
    } else {
        k_update_scalar<E><<<1, 256, 0, st>>>(T, n, h, w);
    }
    return cuda_check(cudaGetLastError(), "update launch");
}

template <typename E>
int launch_expand_update(E *T, uint64_t n, uint64_t hl, uint32_t w, cudaStream_t st) {
    if (n == 0 || (n & (n - 1))) return set_error(TG_ERR_ARG, "table size must be a power of two");
    if (hl >= n) return set_error(TG_ERR_ARG, "expand mask has bits beyond the table");
    const int bits = 63 - __builtin_clzll(n);
    k_expand_update<E><<<grid_for(n >> (bits >= Entry<E>::CB ? Entry<E>::CB : 0), 256), 256, 0, st>>>(T, bits, hl, w);
    return cuda_check(cudaGetLastError(), "expand launch");
}

// in-place select by phases: output block k <- input block 2k+target; for k in [a, 2a) the
// writes lie below block 2a and the reads at or above it (cdist/viterbi.c:149-172)
static int select_inplace(void *T, uint64_t n, int pos, int target, size_t eb, cudaStream_t st) {
    uint64_t blk = 1ull << pos, nb = n >> (pos + 1);
    if (nb == 0) return TG_OK;
    char *B = static_cast<char *>(T);
    const size_t bb = blk * eb;
    if (target) {
        int e = cuda_check(cudaMemcpyAsync(B, B + bb, bb, cudaMemcpyDeviceToDevice, st), "select copy");
        if (e) return e;
    }
    for (uint64_t a = 1; a < nb; a <<= 1) {
        uint64_t hi = std::min(2 * a, nb);
        int e = cuda_check(cudaMemcpy2DAsync(B + a * bb, bb, B + (2 * a + target) * bb, 2 * bb, bb, hi - a,
                                             cudaMemcpyDeviceToDevice, st), "select copy");
        if (e) return e;
    }
    return TG_OK;
}

// ------------------------------------------------------------------ shared-memory tile helpers
// one update over a shared-memory table of 2^bits entries (all threads of the block)
template <typename E>
__device__ __forceinline__ void smem_update(E *T, int bits, uint32_t m, uint32_t w) {
    constexpr int CB = Entry<E>::CB;
    if (bits >= CB && (bits > CB || (m >> CB) == 0)) {
        Chunk *C = reinterpret_cast<Chunk *>(T);
        const uint32_t mhi = m >> CB, mlo = m & ((1u << CB) - 1);
        const uint32_t nch = 1u << (bits - CB);
        if (mhi == 0) {
            for (uint32_t c = threadIdx.x; c < nch; c += blockDim.x) {
                Chunk a = C[c];
                C[c] = chunk_minplus<E>(a, chunk_xor<E>(a, mlo), w);
            }
        } else {
            const int hb = 31 - __clz(mhi);
            // perm(b') = min(perm(b), a + w): both directions from one unpacking of a and perm(b)
            for (uint32_t p = threadIdx.x; p < nch / 2; p += blockDim.x) {
                uint32_t c = insert_zero(p, hb), c2 = c ^ mhi;
                Chunk a = C[c], pb = chunk_xor<E>(C[c2], mlo);
                chunk_minplus_pair<E>(a, pb, w);
                C[c] = a;
                C[c2] = chunk_xor<E>(pb, mlo);
            }
        }
    } else {
        const int hb = 31 - __clz(m);
        const uint32_t n = 1u << bits;
        for (uint32_t p = threadIdx.x; p < n / 2; p += blockDim.x) {
            uint32_t s = insert_zero(p, hb), t = s ^ m;
            E a = T[s], b = T[t];
            T[s] = minplus1<E>(a, b, w);
            T[t] = minplus1<E>(b, a, w);
        }
    }
}

// ------------------------------------------------------------------ single-CTA sweep (narrow tables)
// Op words: bits 30-31 code (0 expand, 1 update, 2 select); update: mask in bits 0-19, weight in
// bits 20-27; select: pos in bits 0-5, target in bit 6.
#define SW_MAXOPS 900
struct SweepParams {
    int nops;
    int w_in;             // width of the input table (0: start from {0: 0})
    int max_bits;         // shared-memory capacity per buffer (entries = 2^max_bits)
    int has_in;
    uint32_t ops[SW_MAXOPS];
};

template <typename E>
__global__ void __launch_bounds__(512) k_sweep_smem(const __grid_constant__ SweepParams P, const E *__restrict__ in,
                                                    E *__restrict__ out) {
    constexpr int CB = Entry<E>::CB;
    extern __shared__ uint4 smem_raw[];
    E *T = reinterpret_cast<E *>(smem_raw);
    E *S = T + (1u << P.max_bits);
    int bits = P.w_in;
    uint32_t n = 1u << bits;
    if (P.has_in) {
        for (uint32_t s = threadIdx.x; s < n; s += blockDim.x) T[s] = in[s];
    } else if (threadIdx.x == 0) {
        T[0] = 0;
    }
    __syncthreads();
    for (int i = 0; i < P.nops; i++) {
        const uint32_t op = P.ops[i];
        const uint32_t code = op >> 30;
        if (code == 0) {
            for (uint32_t s = threadIdx.x; s < n; s += blockDim.x) T[n + s] = (E)Entry<E>::INF;
            bits++;
            n <<= 1;
        } else if (code == 1) {
            smem_update<E>(T, bits, op & 0xFFFFFu, (op >> 20) & 0xFFu);
        } else {
            const int pos = op & 63;
            const uint32_t tgt = (op >> 6) & 1u;
            const uint32_t half = n >> 1;
            if (pos >= CB && half >= (1u << CB)) {
                const Chunk *C = reinterpret_cast<const Chunk *>(T);
                Chunk *D = reinterpret_cast<Chunk *>(S);
                const int cp = pos - CB;
                for (uint32_t q = threadIdx.x; q < (half >> CB); q += blockDim.x)
                    D[q] = C[insert_zero(q, cp) | (tgt << cp)];
            } else {
                for (uint32_t k = threadIdx.x; k < half; k += blockDim.x) S[k] = T[insert_zero(k, pos) | (tgt << pos)];
            }
            E *tmp = T; T = S; S = tmp;
            bits--;
            n >>= 1;
        }
        __syncthreads();
    }
    for (uint32_t s = threadIdx.x; s < n; s += blockDim.x) out[s] = T[s];
}

// ------------------------------------------------------------------ fused tile pass (wide tables)
#define FP_MAXD 20
#define FP_MAXU 48
#define FP_MAXOUTER 64
struct PassParams {
    uint64_t ntiles;
    int d, d_in, d_out, n_outer;
    int nupd, fast_out;
    uint32_t sel_bits;                 // target bits of the selected local bits (smem index)
    uint64_t loc_in[FP_MAXD];          // input entry weight of local bit j (j < d_in)
    uint64_t cmp_out[FP_MAXD];         // output entry weight of compacted local bit j (j < d_out)
    uint32_t cmp_smem[FP_MAXD];        // smem entry weight of compacted local bit j
    uint64_t outer_in[FP_MAXOUTER], outer_out[FP_MAXOUTER];
    uint32_t upd_mask[FP_MAXU];
    uint8_t upd_w[FP_MAXU];
    uint16_t pat[16];                  // smem index of the low compacted entries (generic store)
};

__device__ __forceinline__ uint64_t pdep_w64(uint32_t x, const uint64_t *wt, int nb) {
    uint64_t r = 0;
    for (int j = 0; j < nb; j++)
        if ((x >> j) & 1u) r += wt[j];
    return r;
}
__device__ __forceinline__ uint32_t pdep_w32(uint32_t x, const uint32_t *wt, int nb) {
    uint32_t r = 0;
    for (int j = 0; j < nb; j++)
        if ((x >> j) & 1u) r += wt[j];
    return r;
}

#define FP_THREADS 256
#define FP_TBITS 8

template <typename E>
__global__ void __launch_bounds__(FP_THREADS) k_fused_pass(const __grid_constant__ PassParams P,
                                                          const E *__restrict__ in, E *__restrict__ out) {
    constexpr int CB = Entry<E>::CB;
    extern __shared__ uint4 smem_raw[];
    E *T = reinterpret_cast<E *>(smem_raw);
    Chunk *TC = reinterpret_cast<Chunk *>(smem_raw);
    const uint32_t tid = threadIdx.x;

    // per-thread parts of the chunk address maps (chunk index c = it * FP_THREADS + tid)
    const int nb_in = P.d_in - CB, nb_out = P.d_out - CB;
    const int tb_in = min(nb_in, FP_TBITS), tb_out = min(nb_out, FP_TBITS);
    const uint64_t tid_in = pdep_w64(tid, P.loc_in + CB, tb_in);
    const uint64_t tid_out = pdep_w64(tid, P.cmp_out + CB, tb_out);
    const uint32_t tid_sm = pdep_w32(tid, P.cmp_smem + CB, tb_out);
    const uint32_t nch_in = 1u << nb_in, nch_all = 1u << (P.d - CB), nch_out = 1u << nb_out;

    for (uint64_t tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x) {
        uint64_t ib = 0, ob = 0;
        for (int k = 0; k < P.n_outer; k++)
            if ((tile >> k) & 1ull) { ib += P.outer_in[k]; ob += P.outer_out[k]; }
        // load the input part of the tile, INF over the rows expanded in this pass
        for (uint32_t c = tid; c < nch_in; c += FP_THREADS) {
            uint64_t off = ib + tid_in + pdep_w64(c >> FP_TBITS, P.loc_in + CB + FP_TBITS, nb_in - tb_in);
            cp_async16(TC + c, in + off);
        }
        for (uint32_t c = nch_in + tid; c < nch_all; c += FP_THREADS) {
            Chunk inf;
            inf.w[0] = inf.w[1] = inf.w[2] = inf.w[3] = 0xFFFFFFFFu;
            TC[c] = inf;
        }
        cp_async_wait_all();
        __syncthreads();
        for (int u = 0; u < P.nupd; u++) {
            smem_update<E>(T, P.d, P.upd_mask[u], P.upd_w[u]);
            __syncthreads();
        }
        // store the selected halves in the output layout
        for (uint32_t q = tid; q < nch_out; q += FP_THREADS) {
            const uint32_t qh = q >> FP_TBITS;
            uint64_t off = ob + tid_out + pdep_w64(qh, P.cmp_out + CB + FP_TBITS, nb_out - tb_out);
            uint32_t sidx = tid_sm + pdep_w32(qh, P.cmp_smem + CB + FP_TBITS, nb_out - tb_out) + P.sel_bits;
            Chunk v;
            if (P.fast_out) {
                v = TC[sidx >> CB];
            } else {
                constexpr int PER_WORD = 4 / sizeof(E);
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    uint32_t word = 0;
#pragma unroll
                    for (int e = 0; e < PER_WORD; e++)
                        word |= (uint32_t)T[sidx + P.pat[k * PER_WORD + e]] << (8 * sizeof(E) * e);
                    v.w[k] = word;
                }
            }
            stg_chunk(out + off, v);
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ one op, out of place (wide masks)
// dst = op(src) for an op whose rows do not fit a fused tile: update (code 1), expand (code 0,
// dst holds 2n entries, the upper half INF), select (code 2).
template <typename E>
__global__ void k_single_op(const E *__restrict__ src, E *__restrict__ dst, int bits, int code, uint64_t a, uint32_t b) {
    constexpr int CB = Entry<E>::CB;
    const uint64_t n = 1ull << bits;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const Chunk *S = reinterpret_cast<const Chunk *>(src);
    Chunk *D = reinterpret_cast<Chunk *>(dst);
    if (code == 1) {
        const uint64_t hhi = a >> CB;
        const uint32_t hlo = (uint32_t)(a & ((1u << CB) - 1));
        for (uint64_t c = t0; c < (n >> CB); c += stride)
            stg_chunk(D + c, chunk_minplus<E>(ldg_chunk(S + c), chunk_xor<E>(ldg_chunk(S + (c ^ hhi)), hlo), b));
    } else if (code == 0) {
        Chunk inf;
        inf.w[0] = inf.w[1] = inf.w[2] = inf.w[3] = 0xFFFFFFFFu;
        for (uint64_t c = t0; c < (n >> CB); c += stride) {
            stg_chunk(D + c, ldg_chunk(S + c));
            stg_chunk(D + (n >> CB) + c, inf);
        }
    } else {
        const int pos = (int)a;
        if (pos >= CB) {
            for (uint64_t q = t0; q < (n >> (CB + 1)); q += stride)
                stg_chunk(D + q, ldg_chunk(S + (insert_zero64(q, pos - CB) | ((uint64_t)b << (pos - CB)))));
        } else {
            for (uint64_t k = t0; k < (n >> 1); k += stride) dst[k] = src[insert_zero64(k, pos) | ((uint64_t)b << pos)];
        }
    }
}

// ------------------------------------------------------------------ host scheduler
struct HostOp { int code; uint64_t a; int64_t b; };

struct Seg {
    int kind;               // 0 sweep in shared memory, 1 fused pass, 2 one op out of place
    int op_code = 0;
    uint64_t op_a = 0;
    uint32_t op_b = 0;
    int w_in, w_out;
    int64_t op_end;         // ops done after this segment
    SweepParams sp;
    PassParams pp;
    int ckpt = -1;          // index of a checkpoint written after this segment
};

struct DensePlan {
    int eb;                 // entry bytes
    int peak_bits;
    int64_t nops;
    std::vector<Seg> segs;
    std::vector<int64_t> ckpt_ops;
    int final_buf;          // buffer holding the final table (0: a, 1: b)
    int64_t n_updates;
    double pass_bytes;      // algorithmic bytes moved by the fused passes
    double sweep_bytes;     // bytes read + written by the shared-memory sweeps
};

static int parse_ops(const int64_t *ops, int64_t nops, int eb, std::vector<HostOp> &out, int &peak, int &final_w) {
    out.resize(nops);
    int w = 0;
    peak = 0;
    for (int64_t i = 0; i < nops; i++) {
        HostOp o{(int)ops[3 * i], (uint64_t)ops[3 * i + 1], ops[3 * i + 2]};
        if (o.code == 0) {
            w++;
            if (w > 40) return set_error(TG_ERR_TOO_BIG, "table wider than 40 bits");
        } else if (o.code == 1) {
            if (o.a == 0 || (w < 64 && (o.a >> w) != 0)) return set_error(TG_ERR_ARG, "update mask outside the table");
            uint64_t maxw = eb == 1 ? 254 : 65534;
            if (o.b < 1 || (uint64_t)o.b > maxw) return set_error(TG_ERR_ARG, "column weight out of range");
        } else if (o.code == 2) {
            if ((int64_t)o.a >= w || (o.b != 0 && o.b != 1)) return set_error(TG_ERR_ARG, "bad select op");
            w--;
        } else {
            return set_error(TG_ERR_ARG, "unknown op code");
        }
        peak = std::max(peak, w);
        out[i] = o;
    }
    final_w = w;
    return TG_OK;
}

struct Layout {
    std::vector<int> rows;  // position -> row id
};

// tunables (set by tg_dense_set_tuning)
static int g_dmax8 = 16, g_dmax16 = 15;          // fused tile bits
static int g_sweep_bits8 = 15, g_sweep_bits16 = 14; // shared-memory sweep capacity (bits)

static int build_dense_plan(const int64_t *ops, int64_t nops, int eb, const int64_t *ckpts, int64_t nckpt,
                            DensePlan &P) {
    std::vector<HostOp> hops;
    int peak = 0, final_w = 0;
    int e = parse_ops(ops, nops, eb, hops, peak, final_w);
    if (e) return e;
    if (final_w != 0) return set_error(TG_ERR_ARG, "op stream does not end at width 0");
    const int CB = eb == 1 ? 4 : 3;
    const int DMAX = eb == 1 ? g_dmax8 : g_dmax16;
    const int SWB = eb == 1 ? g_sweep_bits8 : g_sweep_bits16;
    P.eb = eb;
    P.peak_bits = peak;
    P.nops = nops;
    P.n_updates = 0;
    P.pass_bytes = P.sweep_bytes = 0;
    P.ckpt_ops.assign(ckpts, ckpts + nckpt);
    for (auto c : P.ckpt_ops)
        if (c < 0 || c > nops) return set_error(TG_ERR_ARG, "checkpoint outside the op stream");
    std::vector<char> is_ckpt(nops + 1, 0);
    for (auto c : P.ckpt_ops) is_ckpt[c] = 1;

    std::vector<int> active;   // position -> row id
    int next_row = 0;
    int64_t i = 0;
    int buf = 0;
    // a checkpoint at op 0 means the start table {0: 0}: it lives in buffer a (written by the caller)
    while (i < nops) {
        const int w_in = (int)active.size();
        // stop at the next checkpoint
        int64_t limit = nops;
        for (int64_t k = i + 1; k <= nops; k++)
            if (is_ckpt[k]) { limit = k; break; }
        Seg S;
        S.w_in = w_in;
        if (w_in < SWB || (w_in == SWB && hops[i].code != 0)) {
            // shared-memory sweep while the width stays within capacity
            SweepParams &sp = S.sp;
            memset(&sp, 0, sizeof(sp));
            sp.w_in = w_in;
            sp.has_in = i > 0 ? 1 : 0;
            sp.max_bits = SWB;
            int w = w_in;
            int64_t j = i;
            while (j < limit && sp.nops < SW_MAXOPS) {
                const HostOp &o = hops[j];
                if (o.code == 0) {
                    if (w + 1 > SWB) break;
                    sp.ops[sp.nops++] = 0u;
                    active.push_back(next_row++);
                    w++;
                } else if (o.code == 1) {
                    sp.ops[sp.nops++] = (1u << 30) | ((uint32_t)o.b << 20) | (uint32_t)o.a;
                    P.n_updates++;
                } else {
                    sp.ops[sp.nops++] = (2u << 30) | ((uint32_t)o.b << 6) | (uint32_t)o.a;
                    active.erase(active.begin() + o.a);
                    w--;
                }
                j++;
            }
            if (j == i) return set_error(TG_ERR_STATE, "scheduler made no progress");
            S.kind = 0;
            S.w_out = w;
            S.op_end = j;
            P.sweep_bytes += (double)eb * ((sp.has_in ? (1ull << w_in) : 0) + (1ull << w));
            i = j;
        } else {
            // fused pass: grow the run of ops while the tile fits
            const std::vector<int> lin = active;
            auto in_set = [](const std::vector<int> &v, int r) { return std::find(v.begin(), v.end(), r) != v.end(); };
            auto tile_rows = [&](const std::vector<int> &t, const std::vector<int> &lout) {
                std::vector<int> s = t;
                for (int p = 0; p < CB && p < (int)lin.size(); p++) if (!in_set(s, lin[p])) s.push_back(lin[p]);
                for (int p = 0; p < CB && p < (int)lout.size(); p++) if (!in_set(s, lout[p])) s.push_back(lout[p]);
                return s;
            };
            std::vector<int> cur = active, touched;
            int nr = next_row, nupd = 0;
            int64_t j = i;
            while (j < limit && nupd < FP_MAXU) {
                const HostOp &o = hops[j];
                std::vector<int> t2 = touched, cur2 = cur;
                if (o.code == 0) {
                    cur2.push_back(nr);
                    t2.push_back(nr);
                } else if (o.code == 1) {
                    for (int p = 0; p < (int)cur.size(); p++)
                        if (((o.a >> p) & 1ull) && !in_set(t2, cur[p])) t2.push_back(cur[p]);
                } else {
                    if (!in_set(t2, cur[o.a])) t2.push_back(cur[o.a]);
                    cur2.erase(cur2.begin() + o.a);
                }
                if ((int)tile_rows(t2, cur2).size() > DMAX || (int)cur2.size() < CB) break;
                touched.swap(t2);
                cur.swap(cur2);
                if (o.code == 0) nr++;
                else if (o.code == 1) nupd++;
                j++;
            }
            if (j == i) {
                // the op's rows do not fit a tile: one out-of-place pass for it alone
                const HostOp &o = hops[i];
                S.kind = 2;
                S.op_code = o.code;
                S.op_a = o.a;
                S.op_b = (uint32_t)o.b;
                if (o.code == 0) active.push_back(next_row++);
                else if (o.code == 2) active.erase(active.begin() + o.a);
                else P.n_updates++;
                S.w_out = (int)active.size();
                S.op_end = i + 1;
                P.pass_bytes += (double)eb * ((1ull << w_in) + (1ull << S.w_out));
                i = i + 1;
                buf ^= 1;
                if (is_ckpt[S.op_end]) {
                    for (size_t c = 0; c < P.ckpt_ops.size(); c++)
                        if (P.ckpt_ops[c] == S.op_end) { S.ckpt = (int)c; break; }
                }
                P.segs.push_back(S);
                continue;
            }
            // the run's rows: expanded, selected (with targets) and the rows of every update
            std::vector<int> lay = lin;
            std::vector<int> exp_rows, sel_rows, sel_tg;
            std::vector<std::pair<std::vector<int>, int>> upd;
            for (int64_t k = i; k < j; k++) {
                const HostOp &o = hops[k];
                if (o.code == 0) {
                    lay.push_back(next_row);
                    exp_rows.push_back(next_row);
                    next_row++;
                } else if (o.code == 1) {
                    std::vector<int> rr;
                    for (int p = 0; p < (int)lay.size(); p++) if ((o.a >> p) & 1ull) rr.push_back(lay[p]);
                    upd.push_back({rr, (int)o.b});
                    P.n_updates++;
                } else {
                    sel_rows.push_back(lay[o.a]);
                    sel_tg.push_back((int)o.b);
                    lay.erase(lay.begin() + o.a);
                }
            }
            const std::vector<int> &lout = lay;
            std::vector<int> trows = tile_rows(touched, lout);
            // pad with the lowest input positions for larger contiguous loads
            const int w_total = w_in + (int)exp_rows.size();
            int want = std::min(DMAX, std::max((int)trows.size(), std::min(13, w_total - 9)));
            for (int p = 0; p < (int)lin.size() && (int)trows.size() < want; p++)
                if (!in_set(trows, lin[p])) trows.push_back(lin[p]);
            // local order: input rows by input position, then expanded rows in expand order
            std::vector<int> local;
            for (int p = 0; p < (int)lin.size(); p++) if (in_set(trows, lin[p])) local.push_back(lin[p]);
            const int d_in = (int)local.size();
            for (int r : exp_rows) local.push_back(r);
            const int d = (int)local.size();
            if (d > FP_MAXD || d > DMAX) return set_error(TG_ERR_TOO_BIG, "fused tile too large");
            auto local_of = [&](int r) { return (int)(std::find(local.begin(), local.end(), r) - local.begin()); };
            PassParams &pp = S.pp;
            memset(&pp, 0, sizeof(pp));
            pp.d = d;
            pp.d_in = d_in;
            for (int jb = 0; jb < d_in; jb++) {
                int pos = (int)(std::find(lin.begin(), lin.end(), local[jb]) - lin.begin());
                pp.loc_in[jb] = 1ull << pos;
            }
            uint32_t selmask = 0;
            for (size_t k = 0; k < sel_rows.size(); k++) {
                int lb = local_of(sel_rows[k]);
                selmask |= 1u << lb;
                if (sel_tg[k]) pp.sel_bits |= 1u << lb;
            }
            int dout = 0;
            for (int jb = 0; jb < d; jb++) {
                if ((selmask >> jb) & 1u) continue;
                int pos = (int)(std::find(lout.begin(), lout.end(), local[jb]) - lout.begin());
                pp.cmp_out[dout] = 1ull << pos;
                pp.cmp_smem[dout] = 1u << jb;
                dout++;
            }
            pp.d_out = dout;
            // contiguity checks
            for (int jb = 0; jb < CB; jb++) {
                if (pp.loc_in[jb] != (1ull << jb)) return set_error(TG_ERR_STATE, "input tile not contiguous");
                if (pp.cmp_out[jb] != (1ull << jb)) return set_error(TG_ERR_STATE, "output tile not contiguous");
            }
            pp.fast_out = (selmask & ((1u << CB) - 1)) == 0;
            for (int q = 0; q < (1 << CB); q++) {
                uint32_t s = 0;
                for (int jb = 0; jb < CB; jb++) if ((q >> jb) & 1) s += pp.cmp_smem[jb];
                pp.pat[q] = (uint16_t)s;
            }
            // outer rows: input rows outside the tile
            int no = 0;
            for (int p = 0; p < (int)lin.size(); p++) {
                if (in_set(trows, lin[p])) continue;
                if (no >= FP_MAXOUTER) return set_error(TG_ERR_TOO_BIG, "too many outer rows");
                int po = (int)(std::find(lout.begin(), lout.end(), lin[p]) - lout.begin());
                pp.outer_in[no] = 1ull << p;
                pp.outer_out[no] = 1ull << po;
                no++;
            }
            pp.n_outer = no;
            pp.ntiles = 1ull << no;
            pp.nupd = (int)upd.size();
            for (int u = 0; u < pp.nupd; u++) {
                uint32_t m = 0;
                for (int r : upd[u].first) m |= 1u << local_of(r);
                pp.upd_mask[u] = m;
                pp.upd_w[u] = (uint8_t)upd[u].second;
            }
            active = lout;
            S.kind = 1;
            S.w_out = (int)lout.size();
            S.op_end = j;
            P.pass_bytes += (double)eb * ((1ull << w_in) + (1ull << S.w_out));
            i = j;
        }
        buf ^= 1;
        if (is_ckpt[S.op_end]) {
            for (size_t c = 0; c < P.ckpt_ops.size(); c++)
                if (P.ckpt_ops[c] == S.op_end) { S.ckpt = (int)c; break; }
        }
        P.segs.push_back(S);
    }
    P.final_buf = buf;
    return TG_OK;
}

static bool g_attr_done = false;
static int set_attrs() {
    if (g_attr_done) return TG_OK;
    int e;
    e = cuda_check(cudaFuncSetAttribute(k_sweep_smem<uint8_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 << 16), "attr");
    if (e) return e;
    e = cuda_check(cudaFuncSetAttribute(k_sweep_smem<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 << 16), "attr");
    if (e) return e;
    e = cuda_check(cudaFuncSetAttribute(k_fused_pass<uint8_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 1 << 17), "attr");
    if (e) return e;
    e = cuda_check(cudaFuncSetAttribute(k_fused_pass<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, 1 << 17), "attr");
    if (e) return e;
    g_attr_done = true;
    return TG_OK;
}

// resident blocks per SM of a kernel at a block size and dynamic shared memory (cached)
static int resident_blocks(const void *fn, int threads, size_t smem) {
    static std::vector<std::pair<std::pair<const void *, size_t>, int>> cache;
    for (auto &c : cache)
        if (c.first.first == fn && c.first.second == smem) return c.second;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem) != cudaSuccess || n < 1) n = 1;
    cache.push_back({{fn, smem}, n});
    return n;
}

static std::vector<cudaEvent_t> g_events;

static int ensure_events(size_t n) {
    while (g_events.size() < n) {
        cudaEvent_t ev;
        int e = cuda_check(cudaEventCreate(&ev), "event create");
        if (e) return e;
        g_events.push_back(ev);
    }
    return TG_OK;
}

template <typename E>
static int launch_plan(const DensePlan &P, E *a, E *b, void **ckpt_bufs, cudaStream_t st, bool timed = false) {
    int e = set_attrs();
    if (e) return e;
    if (timed && (e = ensure_events(2 * P.segs.size()))) return e;
    E *bufs[2] = {a, b};
    int cur = 0;
    size_t si = 0;
    for (const Seg &S : P.segs) {
        E *src = bufs[cur], *dst = bufs[cur ^ 1];
        if (timed) cudaEventRecord(g_events[2 * si], st);
        if (S.kind == 2) {
            const uint64_t items = ((uint64_t)1 << S.w_in) >> Entry<E>::CB;
            k_single_op<E><<<grid_for(items, 256), 256, 0, st>>>(src, dst, S.w_in, S.op_code, S.op_a, S.op_b);
        } else if (S.kind == 0) {
            size_t sm = 2 * ((size_t)1 << S.sp.max_bits) * sizeof(E);
            k_sweep_smem<E><<<1, 512, sm, st>>>(S.sp, src, dst);
        } else {
            size_t sm = ((size_t)1 << S.pp.d) * sizeof(E);
            int per_sm = resident_blocks((const void *)k_fused_pass<E>, FP_THREADS, sm);
            uint64_t grid = std::min<uint64_t>(S.pp.ntiles, (uint64_t)sm_count() * per_sm);
            k_fused_pass<E><<<(unsigned)grid, FP_THREADS, sm, st>>>(S.pp, src, dst);
        }
        e = cuda_check(cudaGetLastError(), "dense launch");
        if (e) return e;
        if (timed) cudaEventRecord(g_events[2 * si + 1], st);
        si++;
        cur ^= 1;
        if (S.ckpt >= 0 && ckpt_bufs && ckpt_bufs[S.ckpt]) {
            e = cuda_check(cudaMemcpyAsync(ckpt_bufs[S.ckpt], bufs[cur], ((size_t)1 << S.w_out) * sizeof(E),
                                           cudaMemcpyDeviceToDevice, st), "checkpoint copy");
            if (e) return e;
        }
    }
    return TG_OK;
}


// ------------------------------------------------------------------ host emulation (tests only)
// Executes a scheduled plan on host memory with the kernels' own parameters and index
// arithmetic (entry-level arithmetic instead of packed chunks).  Used by the CPU test-suite to
// check the scheduler; the evaluators never call it.
template <typename E>
static void emulate_plan(const DensePlan &P, E *a, E *b, void **ckpt) {
    const int CB = Entry<E>::CB;
    const uint32_t INF = Entry<E>::INF;
    E *bufs[2] = {a, b};
    int cur = 0;
    a[0] = 0;
    for (const Seg &S : P.segs) {
        E *src = bufs[cur], *dst = bufs[cur ^ 1];
        if (S.kind == 2) {
            const uint64_t n = 1ull << S.w_in;
            if (S.op_code == 1) {
                for (uint64_t x = 0; x < n; x++)
                    dst[x] = (E)std::min<uint32_t>(src[x], (uint32_t)src[x ^ S.op_a] + S.op_b);
            } else if (S.op_code == 0) {
                for (uint64_t x = 0; x < n; x++) { dst[x] = src[x]; dst[n + x] = (E)INF; }
            } else {
                const int pos = (int)S.op_a;
                for (uint64_t k = 0; k < n / 2; k++) {
                    uint64_t lo = k & ((1ull << pos) - 1);
                    dst[k] = src[((k ^ lo) << 1) | lo | ((uint64_t)S.op_b << pos)];
                }
            }
        } else if (S.kind == 0) {
            std::vector<E> T;
            if (S.sp.has_in) T.assign(src, src + (1ull << S.sp.w_in));
            else T.assign(1, 0);
            for (int i = 0; i < S.sp.nops; i++) {
                uint32_t op = S.sp.ops[i], code = op >> 30;
                size_t n = T.size();
                if (code == 0) {
                    T.resize(2 * n, (E)INF);
                } else if (code == 1) {
                    uint32_t m = op & 0xFFFFFu, w = (op >> 20) & 0xFFu;
                    int hb = 31 - __builtin_clz(m);
                    for (uint32_t s = 0; s < n; s++) {
                        if ((s >> hb) & 1) continue;
                        uint32_t t = s ^ m;
                        E x = T[s], y = T[t];
                        T[s] = (E)std::min<uint32_t>(x, (uint32_t)y + w);
                        T[t] = (E)std::min<uint32_t>(y, (uint32_t)x + w);
                    }
                } else {
                    int pos = op & 63;
                    uint32_t tgt = (op >> 6) & 1;
                    std::vector<E> U(n / 2);
                    for (uint32_t k = 0; k < n / 2; k++) {
                        uint32_t lo = k & ((1u << pos) - 1);
                        U[k] = T[((k ^ lo) << 1) | lo | (tgt << pos)];
                    }
                    T.swap(U);
                }
            }
            std::copy(T.begin(), T.end(), dst);
        } else {
            const PassParams &pp = S.pp;
            std::vector<E> T((size_t)1 << pp.d);
            for (uint64_t tile = 0; tile < pp.ntiles; tile++) {
                uint64_t ib = 0, ob = 0;
                for (int k = 0; k < pp.n_outer; k++)
                    if ((tile >> k) & 1ull) { ib += pp.outer_in[k]; ob += pp.outer_out[k]; }
                uint32_t nch_in = 1u << (pp.d_in - CB), nch_all = 1u << (pp.d - CB), nch_out = 1u << (pp.d_out - CB);
                for (uint32_t c = 0; c < nch_in; c++) {
                    uint64_t off = ib;
                    for (int j = 0; j < pp.d_in - CB; j++) if ((c >> j) & 1) off += pp.loc_in[CB + j];
                    for (int e = 0; e < (1 << CB); e++) T[((size_t)c << CB) + e] = src[off + e];
                }
                for (uint32_t c = nch_in; c < nch_all; c++)
                    for (int e = 0; e < (1 << CB); e++) T[((size_t)c << CB) + e] = (E)INF;
                for (int u = 0; u < pp.nupd; u++) {
                    uint32_t m = pp.upd_mask[u], w = pp.upd_w[u];
                    int hb = 31 - __builtin_clz(m);
                    for (uint32_t s = 0; s < (1u << pp.d); s++) {
                        if ((s >> hb) & 1) continue;
                        uint32_t t = s ^ m;
                        E x = T[s], y = T[t];
                        T[s] = (E)std::min<uint32_t>(x, (uint32_t)y + w);
                        T[t] = (E)std::min<uint32_t>(y, (uint32_t)x + w);
                    }
                }
                for (uint32_t q = 0; q < nch_out; q++) {
                    uint64_t off = ob;
                    uint32_t sidx = pp.sel_bits;
                    for (int j = 0; j < pp.d_out - CB; j++)
                        if ((q >> j) & 1) { off += pp.cmp_out[CB + j]; sidx += pp.cmp_smem[CB + j]; }
                    for (int e = 0; e < (1 << CB); e++) {
                        uint32_t si = pp.fast_out ? sidx + e : sidx + pp.pat[e];
                        dst[off + e] = T[si];
                    }
                }
            }
        }
        cur ^= 1;
        if (S.ckpt >= 0 && ckpt && ckpt[S.ckpt])
            std::copy(bufs[cur], bufs[cur] + (1ull << S.w_out), static_cast<E *>(ckpt[S.ckpt]));
    }
}

}  // namespace tg

using namespace tg;

// ====================================================================== C-ABI
extern "C" {

int tg_version(void) { return 1; }

const char *tg_last_error(void) { return g_err.c_str(); }

int tg_sm_count(void) { return sm_count(); }

void tg_set_stream(void *stream) { g_stream = static_cast<cudaStream_t>(stream); }

void dp_update(uint8_t *T, uint64_t n, uint64_t h) { launch_update<uint8_t>(T, n, h, 1, cur_stream()); }

void dp_update_w(uint8_t *T, uint64_t n, uint64_t h, int w) {
    if (w < 1 || w > 254) { set_error(TG_ERR_ARG, "weight out of range"); return; }
    launch_update<uint8_t>(T, n, h, (uint32_t)w, cur_stream());
}

void dp_expand_update(uint8_t *T, uint64_t n, uint64_t hl) { launch_expand_update<uint8_t>(T, n, hl, 1, cur_stream()); }

uint64_t dp_select(uint8_t *T, uint64_t n, int pos, int target) {
    if (pos < 0 || (n >> (pos + 1)) == 0) return n;
    select_inplace(T, n, pos, target ? 1 : 0, 1, cur_stream());
    return n >> 1;
}

void dp_fill(uint8_t *T, uint64_t n, uint8_t v) { cuda_check(cudaMemsetAsync(T, v, n, cur_stream()), "fill"); }

void dp_hist(const uint8_t *T, uint64_t n, uint64_t *hist) {
    cudaStream_t st = cur_stream();
    unsigned long long *dh = nullptr;
    if (cuda_check(cudaGetSymbolAddress((void **)&dh, g_hist_dev), "hist symbol")) return;
    if (cuda_check(cudaMemsetAsync(dh, 0, 256 * sizeof(unsigned long long), st), "hist clear")) return;
    k_hist<<<grid_for(n, 256), 256, 0, st>>>(T, n, dh);
    if (cuda_check(cudaGetLastError(), "hist launch")) return;
    if (cuda_check(cudaMemcpyAsync(hist, dh, 256 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st), "hist copy")) return;
    cuda_check(cudaStreamSynchronize(st), "hist sync");
}

int dp_num_threads(void) { return sm_count(); }

// uint16 tables (INF = 65535)
int dp16_update(uint16_t *T, uint64_t n, uint64_t h, int w) {
    if (w < 1 || w > 65534) return set_error(TG_ERR_ARG, "weight out of range");
    return launch_update<uint16_t>(T, n, h, (uint32_t)w, cur_stream());
}
int dp16_expand_update(uint16_t *T, uint64_t n, uint64_t hl, int w) {
    return launch_expand_update<uint16_t>(T, n, hl, (uint32_t)w, cur_stream());
}
uint64_t dp16_select(uint16_t *T, uint64_t n, int pos, int target) {
    if (pos < 0 || (n >> (pos + 1)) == 0) return n;
    select_inplace(T, n, pos, target ? 1 : 0, 2, cur_stream());
    return n >> 1;
}

void *tg_dense_plan(const int64_t *ops, int64_t nops, int entry_bytes, const int64_t *ckpt_ops, int64_t nckpt,
                    int *status) {
    int st = TG_OK;
    DensePlan *P = nullptr;
    if (entry_bytes != 1 && entry_bytes != 2) st = set_error(TG_ERR_ARG, "entry_bytes must be 1 or 2");
    else if (nops < 0 || (nops > 0 && !ops) || nckpt < 0 || (nckpt > 0 && !ckpt_ops)) st = set_error(TG_ERR_ARG, "bad op stream");
    else {
        P = new DensePlan();
        st = build_dense_plan(ops, nops, entry_bytes, ckpt_ops, nckpt, *P);
        if (st) { delete P; P = nullptr; }
    }
    if (status) *status = st;
    return P;
}

int tg_dense_plan_info(void *plan, int64_t *info, int ninfo) {
    if (!plan || !info) return set_error(TG_ERR_ARG, "null plan");
    const DensePlan &P = *static_cast<DensePlan *>(plan);
    int64_t npass = 0, nsweep = 0;
    for (const Seg &S : P.segs) (S.kind ? npass : nsweep)++;   // single-op passes count as passes
    int64_t v[8] = {P.peak_bits, (int64_t)P.segs.size(), npass, nsweep, P.final_buf, P.n_updates,
                    (int64_t)P.pass_bytes, (int64_t)P.sweep_bytes};
    for (int k = 0; k < ninfo && k < 8; k++) info[k] = v[k];
    return TG_OK;
}

int tg_dense_plan_segments(void *plan, int64_t *out, int64_t maxseg) {
    // per segment: kind, w_in, w_out, op_end, tile bits (or sweep capacity), updates in the segment
    if (!plan) return set_error(TG_ERR_ARG, "null plan");
    const DensePlan &P = *static_cast<DensePlan *>(plan);
    int64_t k = 0;
    for (const Seg &S : P.segs) {
        if (k >= maxseg) break;
        out[6 * k + 0] = S.kind;
        out[6 * k + 1] = S.w_in;
        out[6 * k + 2] = S.w_out;
        out[6 * k + 3] = S.op_end;
        out[6 * k + 4] = S.kind == 1 ? S.pp.d : S.kind == 0 ? S.sp.max_bits : -1;
        out[6 * k + 5] = S.kind == 1 ? S.pp.nupd : S.kind == 0 ? S.sp.nops : (S.op_code == 1);
        k++;
    }
    return (int)k;
}

void tg_dense_plan_free(void *plan) { delete static_cast<DensePlan *>(plan); }

int tg_dense_execute(void *plan, void *buf_a, void *buf_b, void **ckpt_bufs, void *stream) {
    if (!plan || !buf_a || !buf_b) return set_error(TG_ERR_ARG, "null plan or buffer");
    const DensePlan &P = *static_cast<DensePlan *>(plan);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the start table {0: 0} in buffer a
    int e;
    if (P.eb == 1) e = cuda_check(cudaMemsetAsync(buf_a, 0, 1, st), "init");
    else e = cuda_check(cudaMemsetAsync(buf_a, 0, 2, st), "init");
    if (e) return e;
    if (P.nops == 0) return TG_OK;
    if (P.eb == 1) return launch_plan<uint8_t>(P, (uint8_t *)buf_a, (uint8_t *)buf_b, ckpt_bufs, st);
    return launch_plan<uint16_t>(P, (uint16_t *)buf_a, (uint16_t *)buf_b, ckpt_bufs, st);
}

int tg_dense_execute_timed(void *plan, void *buf_a, void *buf_b, void *stream, double *out, int nout) {
    // out: per segment kind (0 sweep, 1 fused pass, 2 one-op pass): launches, total ms, bytes
    if (!plan || !buf_a || !buf_b || !out) return set_error(TG_ERR_ARG, "null argument");
    const DensePlan &P = *static_cast<DensePlan *>(plan);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int e = cuda_check(cudaMemsetAsync(buf_a, 0, P.eb, st), "init");
    if (e) return e;
    if (P.eb == 1) e = launch_plan<uint8_t>(P, (uint8_t *)buf_a, (uint8_t *)buf_b, nullptr, st, true);
    else e = launch_plan<uint16_t>(P, (uint16_t *)buf_a, (uint16_t *)buf_b, nullptr, st, true);
    if (e) return e;
    if (P.segs.empty()) return TG_OK;
    e = cuda_check(cudaEventSynchronize(g_events[2 * P.segs.size() - 1]), "event sync");
    if (e) return e;
    double acc[9] = {0};
    for (size_t k = 0; k < P.segs.size(); k++) {
        const Seg &S = P.segs[k];
        float ms = 0.f;
        cudaEventElapsedTime(&ms, g_events[2 * k], g_events[2 * k + 1]);
        int kk = S.kind;
        acc[3 * kk] += 1;
        acc[3 * kk + 1] += ms;
        double bytes = S.kind == 0 ? (double)P.eb * ((S.sp.has_in ? (1ull << S.w_in) : 0) + (1ull << S.w_out))
                                   : (double)P.eb * ((1ull << S.w_in) + (1ull << S.w_out));
        acc[3 * kk + 2] += bytes;
    }
    for (int k = 0; k < nout && k < 9; k++) out[k] = acc[k];
    return TG_OK;
}

int tg_dense_result(void *plan, void *buf_a, void *buf_b, uint32_t *value, void *stream) {
    if (!plan || !value) return set_error(TG_ERR_ARG, "null plan");
    const DensePlan &P = *static_cast<DensePlan *>(plan);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    void *src = P.final_buf ? buf_b : buf_a;
    uint32_t v = 0;
    int e = cuda_check(cudaMemcpyAsync(&v, src, P.eb, cudaMemcpyDeviceToHost, st), "result copy");
    if (e) return e;
    e = cuda_check(cudaStreamSynchronize(st), "result sync");
    if (e) return e;
    *value = v;
    return TG_OK;
}

int tg_dense_run(const int64_t *ops, int64_t nops, int entry_bytes, void *buf_a, void *buf_b, uint32_t *value,
                 void *stream) {
    int st = TG_OK;
    void *P = tg_dense_plan(ops, nops, entry_bytes, nullptr, 0, &st);
    if (!P) return st;
    st = tg_dense_execute(P, buf_a, buf_b, nullptr, stream);
    if (!st) st = tg_dense_result(P, buf_a, buf_b, value, stream);
    tg_dense_plan_free(P);
    return st;
}

int tg_debug_emulate_dense(void *plan, void *host_a, void *host_b, void **ckpt_host) {
    if (!plan || !host_a || !host_b) return set_error(TG_ERR_ARG, "null argument");
    const DensePlan &P = *static_cast<DensePlan *>(plan);
    if (P.eb == 1) emulate_plan<uint8_t>(P, (uint8_t *)host_a, (uint8_t *)host_b, ckpt_host);
    else emulate_plan<uint16_t>(P, (uint16_t *)host_a, (uint16_t *)host_b, ckpt_host);
    return TG_OK;
}

int tg_dense_set_tuning(int dmax8, int dmax16, int sweep_bits8, int sweep_bits16) {
    if (dmax8 < 5 || dmax8 > 17 || dmax16 < 4 || dmax16 > 16 || sweep_bits8 < 4 || sweep_bits8 > 16 ||
        sweep_bits16 < 3 || sweep_bits16 > 15)
        return set_error(TG_ERR_ARG, "tuning out of range");
    g_dmax8 = dmax8; g_dmax16 = dmax16; g_sweep_bits8 = sweep_bits8; g_sweep_bits16 = sweep_bits16;
    return TG_OK;
}

}  // extern "C"
