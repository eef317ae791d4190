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
#include "fused_u8.cuh"
#include "dense_types.cuh"

#include <algorithm>
#include <functional>
#include <cstdio>
#include <cstring>
#include <string>
#include <atomic>
#include <mutex>
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

template <typename E>
__global__ void __launch_bounds__(512) k_sweep_smem(const __grid_constant__ SweepParams P, const E *__restrict__ in,
                                                    E *__restrict__ out) {
    extern __shared__ uint4 smem_raw[];
    sweep_body<E>(P, in, out, smem_raw);
}

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

// uint8 tables: the fused pass with the updates applied in register-resident groups, one persistent
// CTA per SM over a contiguous range of tiles (u8_pass_range).
__global__ void __launch_bounds__(FP_THREADS, 1) k_fused_pass_u8(const __grid_constant__ PassParams P,
                                                                const uint8_t *__restrict__ in,
                                                                uint8_t *__restrict__ out) {
    extern __shared__ uint4 smem_raw[];
    const uint64_t per = P.ntiles / gridDim.x, rem = P.ntiles % gridDim.x;
    const uint64_t t0 = blockIdx.x * per + ((uint64_t)blockIdx.x < rem ? (uint64_t)blockIdx.x : rem);
    const uint64_t t1 = t0 + per + (blockIdx.x < rem ? 1 : 0);
    u8_pass_range(P, t0, t1, in, out, smem_raw);
}

// uint8 one-group passes in the coset-streaming form: one persistent CTA per SM over a contiguous
// range of steps (u8_stream_range).
__global__ void __launch_bounds__(FP_THREADS, 1) k_stream_pass_u8(const __grid_constant__ PassParams P,
                                                                 const uint8_t *__restrict__ in,
                                                                 uint8_t *__restrict__ out) {
    extern __shared__ uint4 smem_raw[];
    // the next pass may be scheduled on an SM as soon as this block leaves it (it waits for the
    // whole grid before touching memory)
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const uint64_t nsteps = (P.ntiles + (1ull << (9 - P.nkt)) - 1) >> (9 - P.nkt);
    const uint64_t per = nsteps / gridDim.x, rem = nsteps % gridDim.x;
    const uint64_t s0 = blockIdx.x * per + ((uint64_t)blockIdx.x < rem ? (uint64_t)blockIdx.x : rem);
    const uint64_t s1 = s0 + per + (blockIdx.x < rem ? 1 : 0);
    u8_stream_range(P, s0, s1, in, out, smem_raw);
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
static int parse_ops(const int64_t *ops, int64_t nops, int eb, std::vector<HostOp> &out, int &peak, int &final_w,
                     int w0 = 0) {
    out.resize(nops);
    int w = w0;
    peak = w0;
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
static bool g_relayout = true;                       // uint8 layout planning between passes
static bool g_cosets = true;                         // coset-streaming form of one-group uint8 passes
static int g_span = 3, g_span_sel = 2;               // streaming passes: update span (4: lane dimension),
                                                     // span when an in-chunk row closes in the pass

// Groups of the pass's updates whose chunk masks (mask >> 4) span <= 3 dimensions, every update
// in a group (the in-chunk part of a mask is free in the register form; see fused_u8.cuh).  Also
// the thread -> coset maps and the store mode.  use_groups = 0 when the register form does not
// apply (tiles of fewer than 7 bits).
static inline bool has_row(const std::vector<int> &v, int r) { return std::find(v.begin(), v.end(), r) != v.end(); }
static inline int index_of(const std::vector<int> &v, int r) { return (int)(std::find(v.begin(), v.end(), r) - v.begin()); }
static inline bool has_bit(const std::vector<int> &v, int b) { return std::find(v.begin(), v.end(), b) != v.end(); }

static void build_groups(PassParams &pp, uint32_t selmask) {
    const int CB = 4;
    (void)selmask;
    pp.use_groups = 0;
    pp.nslow = 0;
    const int nb = pp.d - CB;
    if (nb < 3) return;
    struct G { std::vector<uint32_t> basis; std::vector<int> ups; };
    std::vector<G> gs;
    auto reduce = [](uint32_t v, const std::vector<uint32_t> &basis) {
        for (uint32_t b : basis) {
            int pv = 31 - __builtin_clz(b);
            if ((v >> pv) & 1u) v ^= b;
        }
        return v;
    };
    auto add_vec = [&](std::vector<uint32_t> &basis, uint32_t v) {
        v = reduce(v, basis);
        if (!v) return;
        int pv = 31 - __builtin_clz(v);
        for (uint32_t &b : basis)
            if ((b >> pv) & 1u) b ^= v;
        basis.push_back(v);
    };
    // chunk-level updates first (they shape the bases), then the in-chunk ones into the first group
    for (int pass = 0; pass < 2; pass++) {
        for (int u = 0; u < pp.nupd; u++) {
            const uint32_t c = pp.upd_mask[u] >> CB;
            if ((c == 0) != (pass == 1)) continue;
            bool placed = false;
            for (G &g : gs) {
                if (!reduce(c, g.basis) || g.basis.size() < 3) {
                    add_vec(g.basis, c);
                    g.ups.push_back(u);
                    placed = true;
                    break;
                }
            }
            if (!placed) {
                G g;
                add_vec(g.basis, c);
                g.ups.push_back(u);
                gs.push_back(g);
            }
        }
    }
    if ((int)gs.size() > FP_MAXG) return;
    // store mode from the smem weights of the four lowest output positions
    bool ident = true;
    for (int b = 0; b < CB; b++) ident = ident && pp.cmp_smem[b] == (1u << b);
    pp.store_mode = 2;
    if (ident) {
        pp.store_mode = 0;
    } else {
        for (int sb = 0; sb < CB; sb++) {
            bool ok = true;
            int k = 0;
            for (int b = 0; b <= CB; b++) {
                if (b == sb) continue;
                ok = ok && pp.cmp_smem[k++] == (1u << b);
            }
            if (ok) { pp.store_mode = 1; pp.sel_low = sb; break; }
        }
    }
    int code_i = 0;
    for (size_t gi = 0; gi < gs.size(); gi++) {
        G &g = gs[gi];
        // output chunks from chunk pairs (store mode 1) want chunk bit 0 in the coset
        if (pp.store_mode == 1 && g.basis.size() < 3) add_vec(g.basis, 1u);
        for (int b = nb - 1; b >= 0 && g.basis.size() < 3; b--) add_vec(g.basis, 1u << b);
        std::sort(g.basis.begin(), g.basis.end(), [](uint32_t a, uint32_t b) { return __builtin_clz(a) > __builtin_clz(b); });
        GroupDesc &D = pp.groups[gi];
        memset(&D, 0, sizeof(D));
        uint32_t piv = 0;
        int pv[3];
        for (int j = 0; j < 3; j++) {
            pv[j] = 31 - __builtin_clz(g.basis[j]);
            piv |= 1u << pv[j];
        }
        // coset number -> chunk bits: the three lowest non-pivot bits of distinct residues mod 3
        // first (the lanes of a quarter warp: distinct bank quads under the slot swizzle), then
        // the other non-pivot bits ascending
        std::vector<int> free_bits, order;
        for (int b = 0; b < nb; b++) if (!((piv >> b) & 1u)) free_bits.push_back(b);
        for (int r = 0; r < 3 && (int)order.size() < 3; r++) {
            (void)r;
            for (int b : free_bits) {
                bool clash = false;
                for (int o : order) clash |= (o % 3) == (b % 3);
                if (!clash && !has_bit(order, b)) { order.push_back(b); break; }
            }
        }
        for (int b : free_bits) if (!has_bit(order, b)) order.push_back(b);
        for (size_t j = 0; j < order.size(); j++) D.tpos[j] = (uint8_t)order[j];
        for (int x = 0; x < 8; x++) {
            uint32_t o = 0;
            for (int j = 0; j < 3; j++)
                if ((x >> j) & 1) o ^= g.basis[j];
            D.xoff[x] = o;
        }
        D.first = (uint8_t)code_i;
        D.count = (uint8_t)g.ups.size();
        for (int u : g.ups) {
            const uint32_t m = pp.upd_mask[u], mhi = m >> CB, mlo = m & 15u;
            uint32_t y = 0;
            for (int j = 0; j < 3; j++)
                if ((mhi >> pv[j]) & 1u) y |= 1u << j;
            const uint32_t X = 8 * y + 2 * (mlo >> 2) + (mlo & 1u);
            pp.ucode[code_i] = (uint8_t)(X | (((mlo >> 1) & 1u) << 6));
            pp.uw[code_i] = pp.upd_w[u];
            code_i++;
        }
    }
    pp.ngroups = (int)gs.size();
    pp.use_groups = 1;
}

// The coset-streaming form of a one-group uint8 pass (u8_stream_range): the canonical coset basis
// (the chunk parts of the first independent updates, then extension vectors), the entry
// permutations that make those updates plain member pairings, the residual codes of the other
// updates, the thread -> coset map, the input / output offsets and the store form.  local: tile
// rows (local bit -> row), out: output order, d_in: local bits read from the input.
static void build_stream(PassParams &pp, const std::vector<int> &local, int d_in, const std::vector<int> &out,
                         const std::vector<int> &sel_rows, const std::vector<int> &sel_tg, int w_in, int w_out) {
    const int CB = 4, nb = pp.d - CB;
    pp.stream = 0;
    if (!pp.use_groups || nb < 3 || w_in > 32 || w_out > 32) return;
    if (pp.store_mode == 0) pp.s_mode = 0;
    else if (pp.store_mode == 1) pp.s_mode = 1;
    else return;
    auto reduce = [](uint32_t v, const std::vector<uint32_t> &bs) {     // bs: echelon (distinct top bits)
        for (uint32_t b : bs)
            if ((v ^ b) < v) v ^= b;
        return v;
    };
    auto echelon = [&](const std::vector<uint32_t> &vs) {
        std::vector<uint32_t> e;
        for (uint32_t v : vs) {
            v = reduce(v, e);
            if (v) { e.push_back(v); std::sort(e.begin(), e.end(), std::greater<uint32_t>()); }
        }
        return e;
    };
    // canonical vectors: chunk parts of the first independent updates
    std::vector<uint32_t> B, Bm;
    std::vector<int> Bu, res;
    for (int u = 0; u < pp.nupd; u++) {
        const uint32_t y = pp.upd_mask[u] >> CB;
        if (y && B.size() < 4 && reduce(y, echelon(B))) {
            B.push_back(y);
            Bm.push_back(pp.upd_mask[u] & 15u);
            Bu.push_back(u);
        } else {
            res.push_back(u);
        }
    }
    for (int u : res)
        if (reduce(pp.upd_mask[u] >> CB, echelon(B))) return;          // more than 4 dimensions
    // a fourth dimension goes to the lane pair: a vector other than chunk bit 0, preferably one
    // whose update has no in-chunk part (the straight-line lane update)
    pp.s_lane = 0;
    pp.s_lgen = 0;
    uint32_t LV = 0, LM = 0;
    const bool need_e0 = pp.s_mode == 1 && B.size() == 3 && reduce(1u, echelon(B)) != 0;
    if (B.size() == 4 || need_e0) {
        int jl = -1;
        for (int q = 0; q < 4 && jl < 0; q++) if (B[q] != 1u && Bm[q] == 0) jl = q;
        for (int q = 0; q < 4 && jl < 0; q++) if (B[q] != 1u) jl = q;
        LV = B[jl];
        LM = Bm[jl];
        pp.s_lw = pp.upd_w[Bu[jl]];
        B.erase(B.begin() + jl); Bm.erase(Bm.begin() + jl); Bu.erase(Bu.begin() + jl);
        pp.s_lane = 1;
        pp.s_lgen = LM != 0;
        pp.s_lcode = (uint8_t)((2u * (LM >> 2) + (LM & 1u)) | (((LM >> 1) & 1u) << 6));
    }
    int pb = -1;                        // mode 1: x bit of chunk bit 0 (the pairs of the output chunks)
    std::vector<uint32_t> ext;
    if (pp.s_mode == 1) {
        for (size_t q = 0; q < B.size(); q++)
            if (B[q] == 1u) pb = (int)q;
        if (pb < 0) {
            if (reduce(1u, echelon(B))) {
                if (B.size() == 3) return;
                ext.push_back(1u);
            } else {
                // chunk bit 0 is a sum of canonical vectors: it replaces one of them (whose update
                // becomes residual)
                for (size_t q = 0; q < B.size() && pb < 0; q++) {
                    std::vector<uint32_t> rest;
                    for (size_t r = 0; r < B.size(); r++) if (r != q) rest.push_back(B[r]);
                    rest.push_back(1u);
                    if (echelon(rest).size() == B.size()) {
                        res.push_back(Bu[q]);
                        B.erase(B.begin() + q); Bm.erase(Bm.begin() + q); Bu.erase(Bu.begin() + q);
                        ext.push_back(1u);
                        pb = 0;
                    }
                }
                if (pb < 0) return;
            }
        }
    }
    const int nc = (int)B.size();
    for (uint32_t e : ext) { B.push_back(e); Bm.push_back(0); }
    for (int b = nb - 1; b >= 0 && B.size() < 3; b--) {
        std::vector<uint32_t> cur = B;
        if (pp.s_lane) cur.push_back(LV);
        if (reduce(1u << b, echelon(cur))) { B.push_back(1u << b); Bm.push_back(0); }
    }
    if (B.size() != 3) return;
    if (pp.s_mode == 1)
        for (int q = 0; q < 3; q++) if (B[q] == 1u) pb = q;
    std::vector<uint32_t> BL = B;
    if (pp.s_lane) BL.push_back(LV);
    std::vector<uint32_t> E = echelon(BL);
    if (E.size() != BL.size()) return;
    uint32_t piv = 0, supp = 0;
    for (uint32_t e : E) { piv |= 1u << (31 - __builtin_clz(e)); supp |= e; }
    for (int x = 0; x < 8; x++) {
        uint32_t o = 0, sh = 0;
        for (int j = 0; j < 3; j++)
            if ((x >> j) & 1) { o ^= B[j]; sh ^= Bm[j]; }
        pp.sxoff[x] = o;
        pp.sshift[x] = (uint8_t)sh;
        const uint32_t sp = sh & 1u, shh = (sh >> 1) & 1u;
        auto selu = [&](uint32_t par) { return (par + 2 * shh) | 0x40u | ((par + 2 * (1u - shh)) << 8) | 0x4000u; };
        pp.s_selu[x][0] = selu(sp);
        pp.s_selu[x][1] = selu(1u - sp);
        uint32_t sel = 0;
        for (uint32_t tb = 0; tb < 4; tb++) sel |= (4 * ((tb & 1u) ^ sp) + 2 * (((tb >> 1) & 1u) ^ shh)) << (4 * tb);
        pp.s_selp[x] = sel;
        pp.s_wsw[x] = (uint8_t)(sh >> 2);
    }
    pp.s_nc = nc;
    pp.s_ws = 0;
    for (int x = 0; x < 8; x++) pp.s_ws |= pp.s_wsw[x] != 0;
    for (int q = 0; q < nc; q++) pp.s_cw[q] = pp.upd_w[Bu[q]];
    pp.s_nres = (int)res.size();
    for (size_t q = 0; q < res.size(); q++) {
        const int u = res[q];
        const uint32_t y = pp.upd_mask[u] >> CB, mlo = pp.upd_mask[u] & 15u;
        int c = -1;
        for (int x = 0; x < 8; x++) if (pp.sxoff[x] == y) c = x;
        if (c < 0) return;                 // a residual along the lane dimension: not this form
        const uint32_t r = mlo ^ pp.sshift[c];
        pp.s_rcode[q] = (uint8_t)((8u * c + 2u * (r >> 2) + (r & 1u)) | (((r >> 1) & 1u) << 6));
        pp.s_rw[q] = pp.upd_w[u];
    }
    std::vector<int> opos(pp.d, -1);
    for (int lb = 0; lb < pp.d; lb++) {
        const int q = index_of(out, local[lb]);
        if (q < (int)out.size()) opos[lb] = q;
    }
    auto inw = [&](int b) -> uint64_t { return CB + b < d_in ? pp.loc_in[CB + b] : 0; };
    auto outw = [&](int b) -> uint64_t { return opos[CB + b] >= CB ? (1ull << opos[CB + b]) : 0; };
    uint32_t fixed = 0;
    pp.cfix = pp.selm = pp.selb = pp.expm = 0;
    for (size_t q = 0; q < sel_rows.size(); q++) {
        const int lb = index_of(local, sel_rows[q]);
        const uint32_t t = sel_tg[q] ? 1u : 0u;
        if (lb < CB) {
            if (pp.s_mode != 1 || lb != pp.sel_low) return;
            continue;
        }
        const int b = lb - CB;
        if (!((supp >> b) & 1u)) {
            fixed |= 1u << b;
            pp.cfix |= t << b;
        } else {
            pp.selm |= 1u << b;
            pp.selb |= t << b;
        }
    }
    for (int lb = std::max(d_in, CB); lb < pp.d; lb++) pp.expm |= 1u << (lb - CB);
    // coset-number bits: the free chunk bits, inputs by ascending address (coalesced lanes), then
    // the expanded ones
    std::vector<int> kp;
    for (int b = 0; b < nb; b++)
        if (!((piv >> b) & 1u) && !((fixed >> b) & 1u)) kp.push_back(b);
    std::stable_sort(kp.begin(), kp.end(), [&](int a, int b) {
        const uint64_t wa = inw(a) ? inw(a) : ~0ull, wb = inw(b) ? inw(b) : ~0ull;
        return wa < wb;
    });
    if ((int)kp.size() + pp.s_lane > 9 || (pp.s_lane && kp.size() < 4)) return;
    pp.nk = (int)kp.size();
    pp.nkt = pp.nk + pp.s_lane;
    for (int q = 0; q < pp.nk; q++) {
        pp.kpos[q] = (uint8_t)kp[q];
        pp.kin[q] = (uint32_t)inw(kp[q]);
        pp.kout[q] = (uint32_t)outw(kp[q]);
    }
    for (int x = 0; x < 8; x++) {
        uint64_t a = 0, o = 0;
        for (int b = 0; b < nb; b++)
            if ((pp.sxoff[x] >> b) & 1u) { a ^= inw(b); o ^= outw(b); }
        pp.xin[x] = (uint32_t)a;
        pp.xout[x] = (uint32_t)o;
    }
    uint64_t fa = 0, fo = 0;
    for (int b = 0; b < nb; b++)
        if ((pp.cfix >> b) & 1u) { fa ^= inw(b); fo ^= outw(b); }
    pp.fin = (uint32_t)fa;
    pp.fout = (uint32_t)fo;
    pp.s_lvec = LV;
    uint64_t la = 0, lo = 0;
    for (int b = 0; b < nb; b++)
        if ((LV >> b) & 1u) { la ^= inw(b); lo ^= outw(b); }
    pp.s_lin = (uint32_t)la;
    pp.s_lout = (uint32_t)lo;
    pp.s_pb = pb < 0 ? 0 : pb;
    if (pp.s_mode == 1) {
        const int sb = pp.sel_low;
        const int r = local[sb];
        pp.s_bit = sb;
        pp.s_both = has_row(sel_rows, r) ? 0 : 1;
        pp.s_tgt = 0;
        pp.s_w = 0;
        if (pp.s_both) {
            if (opos[sb] < CB) return;
            pp.s_w = (uint32_t)(1ull << opos[sb]);
        } else {
            pp.s_tgt = sel_tg[index_of(sel_rows, r)] ? 1u : 0u;
        }
    }
    pp.stream = 1;
}

// Row bookkeeping of an op stream: which rows each op touches (rows are numbered in order of
// their expand op), and for each row the ops that update or close it.
struct RowInfo {
    std::vector<std::vector<int>> upd_rows;     // per op: rows of an update
    std::vector<int> sel_row, exp_row;          // per op: row closed / opened (-1)
    std::vector<std::vector<int64_t>> uses;     // per row: ops that update or close it (ascending)
    int64_t next_use(int row, int64_t after) const {
        const auto &u = uses[row];
        auto it = std::lower_bound(u.begin(), u.end(), after);
        return it == u.end() ? INT64_MAX : *it;
    }
};

static void row_info(const std::vector<HostOp> &hops, RowInfo &R, int w0 = 0) {
    const int64_t n = (int64_t)hops.size();
    R.upd_rows.assign(n, {});
    R.sel_row.assign(n, -1);
    R.exp_row.assign(n, -1);
    std::vector<int> canon;
    int next = 0;
    for (; next < w0; next++) {     // rows of the start table
        canon.push_back(next);
        R.uses.emplace_back();
    }
    for (int64_t i = 0; i < n; i++) {
        const HostOp &o = hops[i];
        if (o.code == 0) {
            R.exp_row[i] = next;
            canon.push_back(next++);
            R.uses.emplace_back();
        } else if (o.code == 1) {
            for (int p = 0; p < (int)canon.size(); p++)
                if ((o.a >> p) & 1ull) { R.upd_rows[i].push_back(canon[p]); R.uses[canon[p]].push_back(i); }
        } else {
            R.sel_row[i] = canon[o.a];
            R.uses[canon[o.a]].push_back(i);
            canon.erase(canon.begin() + o.a);
        }
    }
}


int build_dense_plan(const int64_t *ops, int64_t nops, int eb, const int64_t *ckpts, int64_t nckpt,
                     DensePlan &P, int w_start, bool open_end, SegHook on_seg, void *hook_ctx) {
    std::vector<HostOp> hops;
    int peak = 0, final_w = 0;
    if (w_start < 0 || w_start > 40) return set_error(TG_ERR_ARG, "start width out of range");
    int e = parse_ops(ops, nops, eb, hops, peak, final_w, w_start);
    if (e) return e;
    if (final_w != 0 && !open_end) return set_error(TG_ERR_ARG, "op stream does not end at width 0");
    P.w_start = w_start;
    P.final_w = final_w;
    const int CB = eb == 1 ? 4 : 3;
    const int DMAX = eb == 1 ? g_dmax8 : g_dmax16;
    const int SWB = eb == 1 ? g_sweep_bits8 : g_sweep_bits16;
    const bool relayout = eb == 1 && g_relayout;
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
    RowInfo RI;
    row_info(hops, RI, w_start);
    // a segment record is several KB: reserve for about two updates per pass (passes fuse two or
    // more updates; sweeps and relayouts are few) instead of growing by copies
    {
        int64_t nupd = 0;
        for (const HostOp &o : hops) nupd += o.code == 1;
        P.segs.reserve((size_t)std::min<int64_t>(nops + 8, nupd / 2 + 64 + 2 * nckpt));
    }

    std::vector<int> canon;    // canonical order: position -> row (the positions the ops refer to)
    std::vector<int> phys;     // physical order of the table in memory
    for (int r = 0; r < w_start; r++) canon.push_back(r);
    phys = canon;
    int64_t i = 0;
    int buf = 0;
    auto apply_canon = [&](int64_t k, std::vector<int> &c) {
        const HostOp &o = hops[k];
        if (o.code == 0) c.push_back(RI.exp_row[k]);
        else if (o.code == 2) c.erase(c.begin() + o.a);
    };
    auto sweep_next = [&](int w, int64_t k) {       // would a segment starting at op k be a sweep?
        return k < nops && (w < SWB || (w == SWB && hops[k].code != 0));
    };
    auto must_canon = [&](int64_t jend, const std::vector<int> &c) {
        return !relayout || is_ckpt[jend] || jend == nops || sweep_next((int)c.size(), jend);
    };
    // one fused pass over the ops [i0, j0) (possibly none: a relayout to the canonical order)
    auto build_pass = [&](int64_t i0, int64_t j0, const std::vector<int> &touched, bool force_all, Seg &S) -> int {
        const int w_in = (int)canon.size();
        const std::vector<int> lin = phys;
        std::vector<int> inchunk(lin.begin(), lin.begin() + std::min<int>(CB, (int)lin.size()));
            // ---- the run's rows
            std::vector<int> exp_rows, sel_rows, sel_tg;
            std::vector<std::pair<std::vector<int>, int>> upd;
            std::vector<int> cout_ = canon;
            for (int64_t k = i0; k < j0; k++) {
                const HostOp &o = hops[k];
                if (o.code == 0) exp_rows.push_back(RI.exp_row[k]);
                else if (o.code == 1) { upd.push_back({RI.upd_rows[k], (int)o.b}); P.n_updates++; }
                else { sel_rows.push_back(RI.sel_row[k]); sel_tg.push_back((int)o.b); }
                apply_canon(k, cout_);
            }
            const bool force = force_all || must_canon(j0, cout_);
            std::vector<int> trows = touched;
            for (int r : inchunk) if (!has_row(trows, r)) trows.push_back(r);
            if (force)
                for (int p = 0; p < CB && p < (int)cout_.size(); p++)
                    if (!has_row(trows, cout_[p])) trows.push_back(cout_[p]);
            // eviction of one in-chunk row (uint8 layout planning)
            int evict = -1, cand = -1;
            std::vector<int> sel_in;
            for (int r : inchunk) if (has_row(sel_rows, r)) sel_in.push_back(r);
            const bool srule = eb == 1 && g_cosets;
            if (!force && relayout && sel_in.size() <= 1 && (!srule || sel_in.size() == 1)) {
                if (sel_in.size() == 1) {
                    evict = sel_in[0];
                } else {
                    int64_t best = INT64_MAX;
                    const int64_t look = std::max<int64_t>(8, j0 - i0);
                    for (int r : inchunk) {
                        int64_t nu = RI.next_use(r, j0);
                        if (nu < j0 + look && nu < best) { best = nu; evict = r; }
                    }
                }
                if (evict >= 0) {
                    // the input row with the furthest next use enters the in-chunk positions
                    int64_t far = -1;
                    auto consider = [&](int r) {
                        if (has_row(inchunk, r) || has_row(sel_rows, r) || !has_row(lin, r)) return;
                        // streaming form: the row that stays longest (in-chunk rows are free in the
                        // register form); else the row with the furthest next use
                        int64_t nu = srule ? RI.uses[r].empty() ? INT64_MAX : RI.uses[r].back() : RI.next_use(r, j0);
                        if (nu > far) { far = nu; cand = r; }
                    };
                    for (int r : trows) consider(r);
                    if (cand < 0 && (int)trows.size() < DMAX)
                        for (int r : lin) consider(r);
                    if (cand < 0) evict = -1;
                    else if (!has_row(trows, cand)) trows.push_back(cand);
                }
            }
            // pad with the lowest input positions (larger contiguous loads, >= 7 local bits)
            const int w_total = w_in + (int)exp_rows.size();
            int want = std::min(DMAX, std::max((int)trows.size(), std::max(7, w_total - 10)));
            for (int p = 0; p < (int)lin.size() && (int)trows.size() < want; p++)
                if (!has_row(trows, lin[p])) trows.push_back(lin[p]);
            // the four lowest output positions must hold tile rows that survive the pass
            auto survivors = [&]() {
                int n = 0;
                for (int r : trows) n += !has_row(sel_rows, r);
                return n + (int)exp_rows.size() - (int)std::count_if(exp_rows.begin(), exp_rows.end(),
                                                                      [&](int r) { return has_row(trows, r); });
            };
            for (int p = 0; p < (int)lin.size() && survivors() < CB; p++)
                if (!has_row(trows, lin[p])) trows.push_back(lin[p]);
            // local order: in-chunk rows, the entering row, other input rows by input position, expanded rows
            std::vector<int> local(inchunk.begin(), inchunk.end());
            if (cand >= 0) local.push_back(cand);
            for (int r : lin) if (has_row(trows, r) && !has_row(local, r)) local.push_back(r);
            const int d_in = (int)local.size();
            for (int r : exp_rows) local.push_back(r);
            const int d = (int)local.size();
            if (d > FP_MAXD || d > std::max(DMAX, 2 * CB)) return set_error(TG_ERR_TOO_BIG, "fused tile too large");
            // output order
            std::vector<int> out;
            if (force) {
                out = cout_;
            } else {
                std::vector<int> lowrows;
                if (evict >= 0) {
                    for (int b = 0; b <= CB && b < d; b++) if (local[b] != evict) lowrows.push_back(local[b]);
                } else {
                    for (int b = 0; b < CB; b++) if (!has_row(sel_rows, local[b])) lowrows.push_back(local[b]);
                }
                for (int r : lowrows) out.push_back(r);
                for (int r : local) if (!has_row(out, r) && !has_row(sel_rows, r)) out.push_back(r);
                for (int r : lin) if (!has_row(out, r) && !has_row(sel_rows, r)) out.push_back(r);
            }
            if ((int)out.size() != (int)cout_.size()) return set_error(TG_ERR_STATE, "output layout lost a row");
            // the lowest output positions must be tile rows
            for (int p = 0; p < CB && p < (int)out.size(); p++)
                if (!has_row(local, out[p])) return set_error(TG_ERR_STATE, "output chunk rows outside the tile");
            PassParams &pp = S.pp;
            memset(&pp, 0, sizeof(pp));
            pp.d = d;
            pp.d_in = d_in;
            for (int b = 0; b < d_in; b++) pp.loc_in[b] = 1ull << index_of(lin, local[b]);
            uint32_t selmask = 0;
            for (size_t k = 0; k < sel_rows.size(); k++) {
                int lb = index_of(local, sel_rows[k]);
                selmask |= 1u << lb;
                if (sel_tg[k]) pp.sel_bits |= 1u << lb;
            }
            // compacted order = output order of the tile rows
            int dout = 0;
            for (int q = 0; q < (int)out.size(); q++) {
                if (!has_row(local, out[q])) continue;
                pp.cmp_out[dout] = 1ull << q;
                pp.cmp_smem[dout] = 1u << index_of(local, out[q]);
                dout++;
            }
            pp.d_out = dout;
            for (int b = 0; b < CB; b++) {
                if (pp.loc_in[b] != (1ull << b)) return set_error(TG_ERR_STATE, "input tile not contiguous");
                if (pp.cmp_out[b] != (1ull << b)) return set_error(TG_ERR_STATE, "output tile not contiguous");
            }
            bool ident = true;
            for (int b = 0; b < CB; b++) ident = ident && pp.cmp_smem[b] == (1u << b);
            pp.fast_out = ident;
            for (int q = 0; q < (1 << CB); q++) {
                uint32_t sm = 0;
                for (int b = 0; b < CB; b++) if ((q >> b) & 1) sm += pp.cmp_smem[b];
                pp.pat[q] = (uint16_t)sm;
            }
            int no = 0;
            for (int p = 0; p < (int)lin.size(); p++) {
                if (has_row(local, lin[p])) continue;
                if (no >= FP_MAXOUTER) return set_error(TG_ERR_TOO_BIG, "too many outer rows");
                pp.outer_in[no] = 1ull << p;
                pp.outer_out[no] = 1ull << index_of(out, lin[p]);
                no++;
            }
            pp.n_outer = no;
            pp.ntiles = 1ull << no;
            pp.nupd = (int)upd.size();
            for (int u = 0; u < pp.nupd; u++) {
                uint32_t m = 0;
                for (int r : upd[u].first) m |= 1u << index_of(local, r);
                pp.upd_mask[u] = m;
                pp.upd_w[u] = (uint8_t)upd[u].second;
            }
            if (eb == 1) {
                build_groups(pp, selmask);
                if (g_cosets) build_stream(pp, local, d_in, out, sel_rows, sel_tg, w_in, (int)cout_.size());
                // tables that fit L2 together (in + out <= 64 MB) keep their stores cached for the next pass
                pp.s_l2 = ((1ull << w_in) + (1ull << cout_.size())) <= (64ull << 20) ? 1 : 0;
            }
            phys = out;
            canon = cout_;
            S.kind = 1;
            S.w_out = (int)canon.size();
            S.op_end = j0;
            P.pass_bytes += (double)eb * ((1ull << w_in) + (1ull << S.w_out));

        return TG_OK;
    };
    // the first checkpoint after each op (nops when none)
    std::vector<int64_t> next_ckpt(nops + 2, nops);
    for (int64_t k = nops - 1; k >= 0; k--) next_ckpt[k] = is_ckpt[k + 1] ? k + 1 : next_ckpt[k + 1];
    // scratch of the pass-growing loop (assigned per candidate op, no allocation once grown)
    std::vector<int> t2, cur2, need;
    std::vector<uint64_t> b2;
    t2.reserve(64);
    cur2.reserve(64);
    need.reserve(64);
    b2.reserve(64);
    while (i < nops) {
        const int w_in = (int)canon.size();
        const int64_t limit = next_ckpt[i];
        Seg S;
        S.w_in = w_in;
        if (sweep_next(w_in, i) && phys != canon) {
            e = build_pass(i, i, {}, true, S);
            if (e) return e;
        } else if (sweep_next(w_in, i)) {
            SweepParams &sp = S.sp;
            memset(&sp, 0, sizeof(sp));
            sp.w_in = w_in;
            sp.has_in = (i > 0 || w_start > 0) ? 1 : 0;
            sp.max_bits = SWB;
            int w = w_in;
            int64_t j = i;
            while (j < limit && sp.nops < SW_MAXOPS) {
                const HostOp &o = hops[j];
                if (o.code == 0) {
                    if (w + 1 > SWB) break;
                    sp.ops[sp.nops++] = 0u;
                    w++;
                } else if (o.code == 1) {
                    sp.ops[sp.nops++] = (1u << 30) | ((uint32_t)o.b << 20) | (uint32_t)o.a;
                    P.n_updates++;
                } else {
                    sp.ops[sp.nops++] = (2u << 30) | ((uint32_t)o.b << 6) | (uint32_t)o.a;
                    w--;
                }
                apply_canon(j, canon);
                j++;
            }
            if (j == i) return set_error(TG_ERR_STATE, "scheduler made no progress");
            phys = canon;
            S.kind = 0;
            S.w_out = w;
            S.op_end = j;
            P.sweep_bytes += (double)eb * ((sp.has_in ? (1ull << w_in) : 0) + (1ull << w));
            i = j;
        } else {
            // ---- fused pass: grow the run of ops while the tile fits
            const std::vector<int> lin = phys;
            std::vector<int> inchunk(lin.begin(), lin.begin() + std::min<int>(CB, (int)lin.size()));
            std::vector<int> cur = canon, touched;
            int nupd = 0;
            int64_t j = i;
            // coset-streaming passes (uint8): the updates' masks outside the in-chunk rows span at most
            // g_span dimensions (3 in a thread's registers, a 4th across a lane pair), at most one
            // in-chunk row closes, and then at most g_span_sel (the row entering the in-chunk
            // positions joins the coset, in the registers)
            const bool srule = eb == 1 && g_cosets && relayout;
            std::vector<int> srows;                     // row -> bit of the span vectors
            std::vector<uint64_t> sbasis;
            int nsel_in = 0;
            while (j < limit && nupd < FP_MAXU) {
                const HostOp &o = hops[j];
                t2.assign(touched.begin(), touched.end());
                cur2.assign(cur.begin(), cur.end());
                if (o.code == 0) t2.push_back(RI.exp_row[j]);
                else if (o.code == 1) {
                    for (int r : RI.upd_rows[j]) if (!has_row(t2, r)) t2.push_back(r);
                } else if (!has_row(t2, RI.sel_row[j])) t2.push_back(RI.sel_row[j]);
                apply_canon(j, cur2);
                if ((int)cur2.size() < CB) break;
                need.assign(t2.begin(), t2.end());
                for (int r : inchunk) if (!has_row(need, r)) need.push_back(r);
                if (must_canon(j + 1, cur2)) {
                    for (int p = 0; p < CB; p++) if (!has_row(need, cur2[p])) need.push_back(cur2[p]);
                } else if (relayout) {
                    need.push_back(-1);       // room for a row entering the in-chunk positions
                }
                if ((int)need.size() > DMAX) break;
                if (srule) {
                    b2.assign(sbasis.begin(), sbasis.end());
                    int ns2 = nsel_in;
                    if (o.code == 1) {
                        uint64_t v = 0;
                        bool fits = true;
                        for (int r : RI.upd_rows[j]) {
                            if (has_row(inchunk, r)) continue;
                            int q = index_of(srows, r);
                            if (q == (int)srows.size()) {
                                if (q >= 64) { fits = false; break; }
                                srows.push_back(r);
                            }
                            v |= 1ull << q;
                        }
                        if (!fits) break;
                        for (uint64_t b : b2)
                            if ((v ^ b) < v) v ^= b;
                        if (v) {
                            b2.push_back(v);
                            std::sort(b2.begin(), b2.end(), std::greater<uint64_t>());
                        }
                    } else if (o.code == 2 && has_row(inchunk, RI.sel_row[j])) {
                        ns2++;
                    }
                    if (ns2 > 1 || (int)b2.size() > (ns2 ? g_span_sel : g_span)) break;
                    sbasis.swap(b2);
                    nsel_in = ns2;
                }
                touched.swap(t2);
                cur.swap(cur2);
                if (o.code == 1) nupd++;
                j++;
            }
            if (j == i) {
                // the op's rows do not fit a tile: one out-of-place pass on the physical layout
                const HostOp &o = hops[i];
                S.kind = 2;
                S.op_code = o.code;
                S.op_b = (uint32_t)o.b;
                if (o.code == 0) {
                    S.op_a = 0;
                    phys.push_back(RI.exp_row[i]);
                } else if (o.code == 1) {
                    uint64_t m = 0;
                    for (int r : RI.upd_rows[i]) m |= 1ull << index_of(phys, r);
                    S.op_a = m;
                    P.n_updates++;
                } else {
                    int pp_ = index_of(phys, RI.sel_row[i]);
                    S.op_a = (uint64_t)pp_;
                    phys.erase(phys.begin() + pp_);
                }
                apply_canon(i, canon);
                S.w_out = (int)canon.size();
                S.op_end = i + 1;
                P.pass_bytes += (double)eb * ((1ull << w_in) + (1ull << S.w_out));
                i = i + 1;
            } else {
                e = build_pass(i, j, touched, false, S);
                if (e) return e;
                i = j;
            }
        }
        buf ^= 1;
        // checkpoints and the end of a plan that ends with a table are in canonical order
        const bool end_table = open_end && S.op_end == nops;
        if ((is_ckpt[S.op_end] || end_table) && phys != canon) {
            P.segs.push_back(S);
            if (on_seg && (e = on_seg(P.segs.back(), hook_ctx))) return e;
            Seg R;
            R.w_in = (int)canon.size();
            e = build_pass(S.op_end, S.op_end, {}, true, R);
            if (e) return e;
            S = R;
            buf ^= 1;
        }
        if (is_ckpt[S.op_end]) {
            if (phys != canon) return set_error(TG_ERR_STATE, "checkpoint with a non-canonical layout");
            for (size_t c = 0; c < P.ckpt_ops.size(); c++)
                if (P.ckpt_ops[c] == S.op_end) { S.ckpt = (int)c; break; }
        }
        P.segs.push_back(S);
        if (on_seg && (e = on_seg(P.segs.back(), hook_ctx))) return e;
    }
    if (P.segs.capacity() > P.segs.size() + P.segs.size() / 4 + 16) P.segs.shrink_to_fit();
    P.final_buf = buf;
    return TG_OK;
}

static bool g_attr_done = false;
int set_dense_attrs() {
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
    e = cuda_check(cudaFuncSetAttribute(k_fused_pass_u8, cudaFuncAttributeMaxDynamicSharedMemorySize, 3 << 16), "attr");
    if (e) return e;
    e = cuda_check(cudaFuncSetAttribute(k_stream_pass_u8, cudaFuncAttributeMaxDynamicSharedMemorySize, 16 * FS_WARP_BYTES), "attr");
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
static int launch_seg(const Seg &S, E *const bufs[2], int &cur, void **ckpt_bufs, cudaStream_t st, size_t si,
                      bool timed) {
    int e = TG_OK;
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
        if (sizeof(E) == 1 && S.pp.stream) {
            const uint64_t nsteps = (S.pp.ntiles + (1ull << (9 - S.pp.nkt)) - 1) >> (9 - S.pp.nkt);
            const uint64_t grid = std::min<uint64_t>(nsteps, (uint64_t)sm_count());
            // programmatic dependent launch: this pass's blocks start (and run their prologue)
            // while the previous pass drains
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)grid);
            cfg.blockDim = dim3(FP_THREADS);
            cfg.dynamicSmemBytes = 16 * FS_WARP_BYTES;
            cfg.stream = st;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            e = cuda_check(cudaLaunchKernelEx(&cfg, k_stream_pass_u8, S.pp, (const uint8_t *)src, (uint8_t *)dst),
                           "stream pass launch");
            if (e) return e;
        } else if (sizeof(E) == 1 && S.pp.use_groups) {
            // persistent: one CTA per SM, three tile buffers
            uint64_t grid = std::min<uint64_t>(S.pp.ntiles, (uint64_t)sm_count());
            k_fused_pass_u8<<<(unsigned)grid, FP_THREADS, 3 * sm, st>>>(S.pp, (const uint8_t *)src, (uint8_t *)dst);
        } else {
            int per_sm = resident_blocks((const void *)k_fused_pass<E>, FP_THREADS, sm);
            uint64_t grid = std::min<uint64_t>(S.pp.ntiles, (uint64_t)sm_count() * per_sm);
            k_fused_pass<E><<<(unsigned)grid, FP_THREADS, sm, st>>>(S.pp, src, dst);
        }
    }
    e = cuda_check(cudaGetLastError(), "dense launch");
    if (e) return e;
    if (timed) cudaEventRecord(g_events[2 * si + 1], st);
    cur ^= 1;
    if (S.ckpt >= 0 && ckpt_bufs && ckpt_bufs[S.ckpt]) {
        e = cuda_check(cudaMemcpyAsync(ckpt_bufs[S.ckpt], bufs[cur], ((size_t)1 << S.w_out) * sizeof(E),
                                       cudaMemcpyDeviceToDevice, st), "checkpoint copy");
        if (e) return e;
    }
    return TG_OK;
}

template <typename E>
static int launch_plan(const DensePlan &P, E *a, E *b, void **ckpt_bufs, cudaStream_t st, bool timed = false) {
    int e = set_dense_attrs();
    if (e) return e;
    if (timed && (e = ensure_events(2 * P.segs.size()))) return e;
    E *const bufs[2] = {a, b};
    int cur = 0;
    size_t si = 0;
    for (const Seg &S : P.segs) {
        e = launch_seg<E>(S, bufs, cur, ckpt_bufs, st, si++, timed);
        if (e) return e;
    }
    return TG_OK;
}

// launch of every segment as the scheduler emits it (tg_dense_plan_execute)
struct SegLauncher {
    void *bufs[2];
    int cur;
    int eb;
    cudaStream_t st;
};

static int launch_hook(const Seg &S, void *ctx) {
    SegLauncher &Lr = *static_cast<SegLauncher *>(ctx);
    if (Lr.eb == 1) {
        uint8_t *const b[2] = {static_cast<uint8_t *>(Lr.bufs[0]), static_cast<uint8_t *>(Lr.bufs[1])};
        return launch_seg<uint8_t>(S, b, Lr.cur, nullptr, Lr.st, 0, false);
    }
    uint16_t *const b[2] = {static_cast<uint16_t *>(Lr.bufs[0]), static_cast<uint16_t *>(Lr.bufs[1])};
    return launch_seg<uint16_t>(S, b, Lr.cur, nullptr, Lr.st, 0, false);
}

// ------------------------------------------------------------------ host emulation (tests only)
// Executes a scheduled plan on host memory with the kernels' own parameters and index
// arithmetic (entry-level arithmetic instead of packed chunks).  Used by the CPU test-suite to
// check the scheduler; the evaluators never call it.
// the register-group update of k_fused_pass_u8 on host memory: same cosets, register model,
// codes and lane arithmetic as run_group / reg_dispatch
// one update of the register form (reg_dispatch) on an emulated register file
static void emu_reg_update(uint32_t (&R)[64], uint32_t code, uint32_t w) {
    auto sw = [](uint32_t v) { return (v >> 16) | (v << 16); };
    auto addmin = [](uint32_t b, uint32_t w_, uint32_t a) {
        uint32_t lo = std::min((b & 0xFFFFu) + w_, a & 0xFFFFu);
        uint32_t hi = std::min((b >> 16) + w_, a >> 16);
        return lo | (hi << 16);
    };
    const uint32_t X = code & 63u, HS = code >> 6;
    for (uint32_t i = 0; i < 64; i++) {
        const uint32_t j = i ^ X;
        if (X == 0) {
            if (HS) R[i] = addmin(sw(R[i]), w, R[i]);
        } else if (i < j) {
            const uint32_t a = R[i], b = R[j];
            R[i] = addmin(HS ? sw(b) : b, w, a);
            R[j] = addmin(HS ? sw(a) : a, w, b);
        }
    }
}
static void emu_unpack(const uint8_t *ch, uint32_t *R8) {      // one chunk -> R[8x .. 8x + 7]
    for (int wd = 0; wd < 4; wd++) {
        R8[2 * wd] = ch[4 * wd] | ((uint32_t)ch[4 * wd + 2] << 16);
        R8[2 * wd + 1] = ch[4 * wd + 1] | ((uint32_t)ch[4 * wd + 3] << 16);
    }
}
static void emu_pack(const uint32_t *R8, uint8_t *ch) {
    for (int wd = 0; wd < 4; wd++) {
        const uint32_t e = R8[2 * wd], o = R8[2 * wd + 1];
        ch[4 * wd] = (uint8_t)(e & 0xFF);
        ch[4 * wd + 2] = (uint8_t)(e >> 16);
        ch[4 * wd + 1] = (uint8_t)(o & 0xFF);
        ch[4 * wd + 3] = (uint8_t)(o >> 16);
    }
}

static void emulate_groups(const PassParams &pp, uint8_t *T) {
    const int nt = pp.d - 4 - 3;
    const uint32_t ncos = 1u << nt;
    for (int g = 0; g < pp.ngroups; g++) {
        const GroupDesc &G = pp.groups[g];
        for (uint32_t k = 0; k < ncos; k++) {
            uint32_t c0 = 0;
            for (int j = 0; j < nt; j++) c0 |= ((k >> j) & 1u) << G.tpos[j];
            uint32_t R[64];
            for (int x = 0; x < 8; x++) emu_unpack(T + 16 * (size_t)(c0 ^ G.xoff[x]), R + 8 * x);
            for (int u = 0; u < G.count; u++) emu_reg_update(R, pp.ucode[G.first + u], pp.uw[G.first + u]);
            for (int x = 0; x < 8; x++) emu_pack(R + 8 * x, T + 16 * (size_t)(c0 ^ G.xoff[x]));
        }
    }
}

// the coset-streaming pass (u8_stream_range) on host memory: the same steps, coset map, entry
// permutations, update codes, offsets and store forms, thread by thread
static void emulate_stream(const PassParams &pp, const uint8_t *src, uint8_t *dst) {
    const int g = 9 - pp.nkt;
    const int ng = std::min(g, pp.n_outer);
    const uint64_t nsteps = (pp.ntiles + (1ull << g) - 1) >> g;
    auto reg = [](int x, uint32_t q) { return 8 * x + 2 * (int)(q >> 2) + (int)(q & 1u); };
    auto sw = [](uint32_t v) { return (v >> 16) | (v << 16); };
    auto addmin = [](uint32_t b, uint32_t w_, uint32_t a) {
        uint32_t lo = std::min((b & 0xFFFFu) + w_, a & 0xFFFFu);
        uint32_t hi = std::min((b >> 16) + w_, a >> 16);
        return lo | (hi << 16);
    };
    std::vector<uint32_t> RA((size_t)FP_THREADS * 64);
    std::vector<uint32_t> C0(FP_THREADS), OUTC(FP_THREADS);
    std::vector<uint64_t> OB(FP_THREADS);
    std::vector<char> VALID(FP_THREADS);
    for (uint64_t s = 0; s < nsteps; s++) {
        for (uint32_t tid = 0; tid < FP_THREADS; tid++) {
            const uint32_t k = tid & ((1u << pp.nkt) - 1u), j = tid >> pp.nkt;
            VALID[tid] = ((s << g) | j) < pp.ntiles;
            if (!VALID[tid]) continue;
            uint32_t c0 = pp.cfix, inc = pp.fin, outc = pp.fout;
            for (int q = 0; q < pp.nk; q++) {
                const int bit = (pp.s_lane && q >= 4) ? q + 1 : q;
                if ((k >> bit) & 1u) { c0 ^= 1u << pp.kpos[q]; inc ^= pp.kin[q]; outc ^= pp.kout[q]; }
            }
            if (pp.s_lane && ((k >> 4) & 1u)) { c0 ^= pp.s_lvec; inc ^= pp.s_lin; outc ^= pp.s_lout; }
            uint64_t ib = 0, ob = 0;
            for (int q = 0; q < ng; q++)
                if ((j >> q) & 1u) { ib += pp.outer_in[q]; ob += pp.outer_out[q]; }
            for (int q = ng; q < pp.n_outer; q++)
                if ((s >> (q - ng)) & 1ull) { ib += pp.outer_in[q]; ob += pp.outer_out[q]; }
            uint32_t *R = &RA[(size_t)tid * 64];
            std::fill(R, R + 64, 0u);
            for (int x = 0; x < 8; x++) {
                const uint32_t c = c0 ^ pp.sxoff[x];
                uint8_t ch[16];
                if (c & pp.expm) memset(ch, 0xFF, 16);
                else memcpy(ch, src + ib + (inc ^ pp.xin[x]), 16);
                for (uint32_t q = 0; q < 16; q++)       // storage position q holds entry q ^ shift
                    R[reg(x, q)] |= (uint32_t)ch[q ^ pp.sshift[x]] << (16 * ((q >> 1) & 1u));
            }
            uint32_t (&Rr)[64] = *reinterpret_cast<uint32_t(*)[64]>(R);
            for (int u = 0; u < pp.s_nres; u++) emu_reg_update(Rr, pp.s_rcode[u], pp.s_rw[u]);
            for (int u = 0; u < pp.s_nc; u++) emu_reg_update(Rr, 8u << u, pp.s_cw[u]);
            C0[tid] = c0;
            OUTC[tid] = outc;
            OB[tid] = ob;
        }
        if (pp.s_lane) {                 // the lane update: pairs (tid, tid ^ 16) from the old values
            const uint32_t X = pp.s_lcode & 63u, HS = pp.s_lcode >> 6;
            std::vector<uint32_t> old(RA);
            for (uint32_t tid = 0; tid < FP_THREADS; tid++) {
                if (!VALID[tid]) continue;
                const uint32_t *P2 = &old[(size_t)(tid ^ 16u) * 64];
                uint32_t *R = &RA[(size_t)tid * 64];
                for (uint32_t i = 0; i < 64; i++) {
                    const uint32_t v = P2[i ^ X];
                    R[i] = addmin(HS ? sw(v) : v, pp.s_lw, old[(size_t)tid * 64 + i]);
                }
            }
        }
        for (uint32_t tid = 0; tid < FP_THREADS; tid++) {
            if (!VALID[tid]) continue;
            const uint32_t *R = &RA[(size_t)tid * 64];
            const uint32_t c0 = C0[tid], outc = OUTC[tid];
            const uint64_t ob = OB[tid];
            uint8_t W[8][16];
            for (int x = 0; x < 8; x++)
                for (uint32_t e = 0; e < 16; e++) {
                    const uint32_t q = e ^ pp.sshift[x];
                    W[x][e] = (uint8_t)(R[reg(x, q)] >> (16 * ((q >> 1) & 1u)));
                }
            const int PB = 1 << pp.s_pb;
            for (int x = 0; x < 8; x++) {
                const uint32_t c = c0 ^ pp.sxoff[x];
                if ((c & pp.selm) != pp.selb) continue;
                if (pp.s_mode == 0) {
                    memcpy(dst + ob + (outc ^ pp.xout[x]), W[x], 16);
                } else if (!(x & PB)) {
                    const int sb = pp.s_bit;
                    const bool swp = (pp.sxoff[x] ^ c0) & 1u;
                    const uint8_t *A = swp ? W[x | PB] : W[x], *B = swp ? W[x] : W[x | PB];
                    for (uint32_t t = 0; t < 2; t++) {
                        if (!pp.s_both && t != pp.s_tgt) continue;
                        uint8_t *o = dst + ob + (outc ^ pp.xout[x]) + (pp.s_both ? t * pp.s_w : 0);
                        for (uint32_t e = 0; e < 16; e++) {
                            const uint32_t lo = e & ((1u << sb) - 1);
                            const uint32_t se = ((e ^ lo) << 1) | lo | (t << sb);
                            o[e] = se < 16 ? A[se] : B[se - 16];
                        }
                    }
                }
            }
        }
    }
}

template <typename E>
static void emulate_plan(const DensePlan &P, E *a, E *b, void **ckpt) {
    const int CB = Entry<E>::CB;
    const uint32_t INF = Entry<E>::INF;
    E *bufs[2] = {a, b};
    int cur = 0;
    if (P.w_start == 0) a[0] = 0;      // a plan from a given table finds it in a
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
            if (sizeof(E) == 1 && pp.stream)
                emulate_stream(pp, reinterpret_cast<const uint8_t *>(src), reinterpret_cast<uint8_t *>(dst));
            else for (uint64_t tile = 0; tile < pp.ntiles; tile++) {
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
                const bool groups = sizeof(E) == 1 && pp.use_groups;
                if (groups) {
                    emulate_groups(pp, reinterpret_cast<uint8_t *>(T.data()));
                    for (int u2 = 0; u2 < pp.nslow; u2++) {
                        const int k2 = pp.slow_idx[u2];
                        uint32_t m = pp.upd_mask[k2], w = pp.upd_w[k2];
                        int hb = 31 - __builtin_clz(m);
                        for (uint32_t s = 0; s < (1u << pp.d); s++) {
                            if ((s >> hb) & 1) continue;
                            uint32_t t = s ^ m;
                            E x = T[s], y = T[t];
                            T[s] = (E)std::min<uint32_t>(x, (uint32_t)y + w);
                            T[t] = (E)std::min<uint32_t>(y, (uint32_t)x + w);
                        }
                    }
                } else {
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
                }
                for (uint32_t q = 0; q < nch_out; q++) {
                    uint64_t off = ob;
                    uint32_t sidx = pp.sel_bits;
                    for (int j = 0; j < pp.d_out - CB; j++)
                        if ((q >> j) & 1) { off += pp.cmp_out[CB + j]; sidx += pp.cmp_smem[CB + j]; }
                    if (groups && pp.store_mode == 1) {
                        // output entry e <- the 32-entry span without local bit sel_low (value t)
                        const int sb = pp.sel_low;
                        const uint32_t t = (sidx >> sb) & 1u, base = (sidx >> 5) << 5;
                        for (uint32_t e = 0; e < 16; e++) {
                            uint32_t lo = e & ((1u << sb) - 1);
                            uint32_t src_e = ((e ^ lo) << 1) | lo | (t << sb);
                            dst[off + e] = T[base + src_e];
                        }
                        continue;
                    }
                    const bool fast = groups ? pp.store_mode == 0 : pp.fast_out;
                    for (int e = 0; e < (1 << CB); e++) {
                        uint32_t si = fast ? sidx + e : sidx + pp.pat[e];
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

// ------------------------------------------------------------------ allocation-free entry point
// Some callers cannot allocate device memory: a runtime that owns the whole device-memory budget
// and hands out only the buffers it planned for (a serving engine's pool, another framework's
// arena), or a caller on a latency-critical stream where cudaMalloc / cudaFree would synchronize
// the device and stall concurrent work.  For them, tg_dense_run_noalloc runs a whole plan with
// the second (ping-pong) table in this file-scope array instead of a caller-provided buffer.  Every
// GPU that loads the library holds the array until the process exits.
#define TG_NOALLOC_MAX_BITS 22
static __device__ __align__(256) uint8_t g_noalloc_scratch[1u << TG_NOALLOC_MAX_BITS];
#define TG_NOALLOC_MAX_DEVICES 64
static std::atomic<uint8_t *> g_noalloc_ptr[TG_NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mu;

// device address of the scratch array on the current device (looked up once per device, under a
// lock so that two host threads making their first call at once agree; the array's name in host
// code is only a stand-in, not an address a kernel may use)
static int noalloc_scratch(uint8_t **out) {
    int dev = 0;
    int e = cuda_check(cudaGetDevice(&dev), "get device");
    if (e) return e;
    if (dev < 0 || dev >= TG_NOALLOC_MAX_DEVICES) return set_error(TG_ERR_TOO_BIG, "device index beyond the table");
    uint8_t *p = g_noalloc_ptr[dev].load(std::memory_order_acquire);
    if (!p) {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        p = g_noalloc_ptr[dev].load(std::memory_order_relaxed);
        if (!p) {
            void *q = nullptr;
            e = cuda_check(cudaGetSymbolAddress(&q, g_noalloc_scratch), "scratch symbol address");
            if (e) return e;
            p = static_cast<uint8_t *>(q);
            g_noalloc_ptr[dev].store(p, std::memory_order_release);
        }
    }
    *out = p;
    return TG_OK;
}


// ------------------------------------------------------------------ witness of a small plan
// One block applies the ops one after another, keeping every table of the sweep (T_0 = {0: 0},
// T_k+1 = op_k(T_k)) one after another in `tabs`; then one thread walks back from the final entry:
// a select restores its bit, an update whose table before it does not hold the current value at
// the current state was used (the state moves by its mask, the value drops by its weight), the
// traceback of the reference's auto.py.  out: [0] final entry, [1] number of used updates, [2..]
// their op indices (last op first), [2 + out_cap] status (0 ok, 1 storage or op out of range, 2
// traceback lost the path).
template <typename E>
__global__ void __launch_bounds__(1024) k_witness_small(const int64_t *ops, int64_t n, E *tabs, uint64_t cap,
                                                        int32_t *out, int64_t out_cap) {
    constexpr uint32_t INF = Entry<E>::INF;
    const unsigned tid = threadIdx.x, NT = blockDim.x;
    uint64_t off = 0;
    int w = 0;
    if (tid == 0) tabs[0] = 0;
    __syncthreads();
    for (int64_t k = 0; k < n; k++) {
        const int code = (int)ops[3 * k];
        const uint64_t a = (uint64_t)ops[3 * k + 1];
        const int64_t b = ops[3 * k + 2];
        const int w2 = code == 0 ? w + 1 : code == 2 ? w - 1 : w;
        const uint64_t m = 1ull << w, m2 = 1ull << (w2 < 0 ? 0 : w2);
        const bool bad = w2 < 0 || w2 > 30 || off + m + m2 > cap || (code == 1 && (a >> w)) ||
                         (code == 2 && (a >= (uint64_t)w || b < 0 || b > 1)) || code < 0 || code > 2 ||
                         (code == 1 && (b < 1 || b > (int64_t)INF));
        if (bad) {
            if (tid == 0) out[2 + out_cap] = 1;
            return;
        }
        const E *S = tabs + off;
        E *D = tabs + off + m;
        if (code == 0) {
            for (uint64_t i = tid; i < m; i += NT) {
                D[i] = S[i];
                D[i + m] = (E)INF;
            }
        } else if (code == 1) {
            for (uint64_t i = tid; i < m; i += NT) {
                const uint32_t x = S[i], y = S[i ^ a];
                const uint32_t c = y == INF ? INF : min(y + (uint32_t)b, INF);
                D[i] = (E)min(x, c);
            }
        } else {
            const uint64_t low = (1ull << a) - 1ull;
            for (uint64_t i = tid; i < m2; i += NT)
                D[i] = S[((i & ~low) << 1) | ((uint64_t)b << a) | (i & low)];
        }
        off += m;
        w = w2;
        __syncthreads();
    }
    if (tid != 0) return;
    const uint32_t value = tabs[off];
    out[0] = (int32_t)value;
    int64_t used = 0;
    int status = 0;
    if (w == 0 && value != INF) {
        uint64_t st = 0;
        uint32_t v = value;
        for (int64_t k = n - 1; k >= 0; k--) {
            const int code = (int)ops[3 * k];
            const uint64_t a = (uint64_t)ops[3 * k + 1];
            const int64_t b = ops[3 * k + 2];
            const int wb = code == 0 ? w - 1 : code == 2 ? w + 1 : w;      // width before op k
            off -= 1ull << wb;
            if (code == 2) {
                const uint64_t low = (1ull << a) - 1ull;
                st = ((st & ~low) << 1) | ((uint64_t)b << a) | (st & low);
            } else if (code == 0) {
                if (st >> wb) { status = 2; break; }
            } else if (tabs[off + st] != v) {
                st ^= a;
                v -= (uint32_t)b;
                if (tabs[off + st] != v) { status = 2; break; }
                if (used < out_cap) out[2 + used] = (int32_t)k;
                used++;
            }
            w = wb;
        }
        if (!status && (st != 0 || v != 0)) status = 2;
    } else if (w != 0) {
        status = 1;
    }
    out[1] = (int32_t)used;
    out[2 + out_cap] = status;
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

// tg_dense_plan + tg_dense_execute in one call, each segment launched on `stream` as soon as it is
// scheduled, so the first passes run while the rest of the plan is scheduled; returns the plan
// (for tg_dense_result / tg_dense_plan_info / tg_dense_plan_free).  Buffers as tg_dense_execute
// (2^peak_bits entries each).  On an error the launches made so far stay queued.
void *tg_dense_plan_execute(const int64_t *ops, int64_t nops, int entry_bytes, void *buf_a, void *buf_b,
                            uint64_t buf_entries, void *stream, int *status) {
    int st = TG_OK;
    DensePlan *P = nullptr;
    // the widest table of the op stream, before anything is launched
    int64_t w = 0, peak = 0;
    for (int64_t k = 0; ops && k < nops; k++) {
        w += ops[3 * k] == 0 ? 1 : ops[3 * k] == 2 ? -1 : 0;
        peak = std::max(peak, w);
    }
    if (entry_bytes != 1 && entry_bytes != 2) st = set_error(TG_ERR_ARG, "entry_bytes must be 1 or 2");
    else if (nops < 0 || (nops > 0 && !ops) || !buf_a || !buf_b) st = set_error(TG_ERR_ARG, "bad op stream or buffer");
    else if (peak > 40 || (1ull << peak) > buf_entries) st = set_error(TG_ERR_ARG, "buffers smaller than 2^peak_bits");
    else if ((st = set_dense_attrs()) == TG_OK) {
        SegLauncher Lr;
        Lr.bufs[0] = buf_a;
        Lr.bufs[1] = buf_b;
        Lr.cur = 0;
        Lr.eb = entry_bytes;
        Lr.st = static_cast<cudaStream_t>(stream);
        st = cuda_check(cudaMemsetAsync(buf_a, 0, entry_bytes, Lr.st), "init");
        if (!st) {
            P = new DensePlan();
            st = build_dense_plan(ops, nops, entry_bytes, nullptr, 0, *P, 0, false, launch_hook, &Lr);
            if (st) { delete P; P = nullptr; }
        }
    }
    if (status) *status = st;
    return P;
}

// A plan of the ops that follow a table of width w_start (canonical order, given by the caller in
// buffer a at execution); it may end at any width, with its final table in canonical order.
// For recomputing segments of a sweep from a checkpoint (the witness traceback).
void *tg_dense_plan_from(const int64_t *ops, int64_t nops, int entry_bytes, int w_start, const int64_t *ckpt_ops,
                         int64_t nckpt, int *status) {
    int st = TG_OK;
    DensePlan *P = nullptr;
    if (entry_bytes != 1 && entry_bytes != 2) st = set_error(TG_ERR_ARG, "entry_bytes must be 1 or 2");
    else if (nops < 0 || (nops > 0 && !ops) || nckpt < 0 || (nckpt > 0 && !ckpt_ops)) st = set_error(TG_ERR_ARG, "bad op stream");
    else {
        P = new DensePlan();
        st = build_dense_plan(ops, nops, entry_bytes, ckpt_ops, nckpt, *P, w_start, true);
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
    // per segment: kind, w_in, w_out, op_end, tile bits (or sweep capacity), updates in the segment,
    // register groups (0: shared-memory updates), store mode
    if (!plan) return set_error(TG_ERR_ARG, "null plan");
    const DensePlan &P = *static_cast<DensePlan *>(plan);
    int64_t k = 0;
    for (const Seg &S : P.segs) {
        if (k >= maxseg) break;
        int64_t *o = out + 8 * k;
        o[0] = S.kind == 1 && S.pp.stream ? 3 : S.kind;
        o[1] = S.w_in;
        o[2] = S.w_out;
        o[3] = S.op_end;
        o[4] = S.kind == 1 ? S.pp.d : S.kind == 0 ? S.sp.max_bits : -1;
        o[5] = S.kind == 1 ? S.pp.nupd : S.kind == 0 ? S.sp.nops : (S.op_code == 1);
        if (S.kind == 1 && S.pp.stream) {
            int ws = 0;
            for (int x = 0; x < 8; x++) ws |= S.pp.s_wsw[x] != 0;
            o[6] = S.pp.s_nres + 16 * ws + 32 * S.pp.s_lane + 64 * S.pp.s_lgen;
        } else {
            o[6] = S.kind == 1 && S.pp.use_groups ? S.pp.ngroups : 0;
        }
        o[7] = S.kind == 1 ? S.pp.store_mode : -1;
        k++;
    }
    return (int)k;
}

void tg_dense_plan_free(void *plan) { delete static_cast<DensePlan *>(plan); }

int tg_dense_segment_ms(void *plan, float *out, int64_t maxseg) {
    if (!plan || !out) return set_error(TG_ERR_ARG, "null argument");
    const DensePlan &P = *static_cast<DensePlan *>(plan);
    int64_t k = 0;
    for (; k < maxseg && k < (int64_t)P.seg_ms.size(); k++) out[k] = P.seg_ms[k];
    return (int)k;
}

int tg_dense_execute(void *plan, void *buf_a, void *buf_b, void **ckpt_bufs, void *stream) {
    if (!plan || !buf_a || !buf_b) return set_error(TG_ERR_ARG, "null plan or buffer");
    const DensePlan &P = *static_cast<DensePlan *>(plan);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the start table {0: 0} in buffer a (a plan from a given table finds it there)
    int e = TG_OK;
    if (P.w_start == 0) e = cuda_check(cudaMemsetAsync(buf_a, 0, P.eb, st), "init");
    if (e) return e;
    if (P.nops == 0) return TG_OK;
    if (P.eb == 1) return launch_plan<uint8_t>(P, (uint8_t *)buf_a, (uint8_t *)buf_b, ckpt_bufs, st);
    return launch_plan<uint16_t>(P, (uint16_t *)buf_a, (uint16_t *)buf_b, ckpt_bufs, st);
}

int tg_dense_execute_timed(void *plan, void *buf_a, void *buf_b, void *stream, double *out, int nout) {
    // out: per segment kind (0 sweep, 1 fused tile pass, 2 one-op pass, 3 coset-streaming pass):
    // launches, total ms, bytes
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
    double acc[12] = {0};
    DensePlan &PM = *static_cast<DensePlan *>(plan);
    PM.seg_ms.assign(P.segs.size(), 0.f);
    for (size_t k = 0; k < P.segs.size(); k++) {
        const Seg &S = P.segs[k];
        float ms = 0.f;
        cudaEventElapsedTime(&ms, g_events[2 * k], g_events[2 * k + 1]);
        PM.seg_ms[k] = ms;
        const int kk = S.kind == 1 && S.pp.stream ? 3 : S.kind;
        acc[3 * kk] += 1;
        acc[3 * kk + 1] += ms;
        double bytes = S.kind == 0 ? (double)P.eb * ((S.sp.has_in ? (1ull << S.w_in) : 0) + (1ull << S.w_out))
                                   : (double)P.eb * ((1ull << S.w_in) + (1ull << S.w_out));
        acc[3 * kk + 2] += bytes;
    }
    for (int k = 0; k < nout && k < 12; k++) out[k] = acc[k];
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

int tg_dense_run_noalloc(const int64_t *ops, int64_t nops, uint8_t *table_dev, uint64_t table_entries,
                         uint32_t *value, void *stream) {
    if (!value || (nops > 0 && !ops) || nops < 0) return set_error(TG_ERR_ARG, "bad op stream or result pointer");
    if (!table_dev) return set_error(TG_ERR_ARG, "null table");
    DensePlan P;
    int e = build_dense_plan(ops, nops, 1, nullptr, 0, P);
    if (e) return e;
    if (P.peak_bits > TG_NOALLOC_MAX_BITS)
        return set_error(TG_ERR_TOO_BIG, "plan wider than the 2^22-entry scratch of tg_dense_run_noalloc");
    if (table_entries < (1ull << P.peak_bits)) return set_error(TG_ERR_ARG, "table buffer smaller than 2^peak_bits");
    uint8_t *scratch = nullptr;
    e = noalloc_scratch(&scratch);
    if (e) return e;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the start table {0: 0} is the first entry of the caller's table; the scratch needs no
    // clearing: every launch writes its whole output table before anything reads it
    e = cuda_check(cudaMemsetAsync(table_dev, 0, 1, st), "init");
    if (e) return e;
    if (nops > 0) {
        e = launch_plan<uint8_t>(P, table_dev, scratch, nullptr, st);
        if (e) return e;
    }
    uint32_t v = 0;
    e = cuda_check(cudaMemcpyAsync(&v, P.final_buf ? scratch : table_dev, 1, cudaMemcpyDeviceToHost, st), "result copy");
    if (e) return e;
    e = cuda_check(cudaStreamSynchronize(st), "result sync");
    if (e) return e;
    *value = v;
    return TG_OK;
}

// Update span of the coset-streaming passes (3: a thread's registers; 4: with the lane
// dimension), and the span when an in-chunk row closes in the pass (2 or 3).
int tg_dense_set_stream_span(int span, int span_sel) {
    if (span < 2 || span > 4 || span_sel < 1 || span_sel > 3 || span_sel > span)
        return set_error(TG_ERR_ARG, "stream span out of range");
    g_span = span;
    g_span_sel = span_sel;
    return TG_OK;
}

int tg_dense_set_tuning(int dmax8, int dmax16, int sweep_bits8, int sweep_bits16) {
    if (dmax8 < 5 || dmax8 > 16 || dmax16 < 4 || dmax16 > 16 || sweep_bits8 < 4 || sweep_bits8 > 16 ||
        sweep_bits16 < 3 || sweep_bits16 > 15)
        return set_error(TG_ERR_ARG, "tuning out of range");
    g_dmax8 = dmax8; g_dmax16 = dmax16; g_sweep_bits8 = sweep_bits8; g_sweep_bits16 = sweep_bits16;
    return TG_OK;
}


// bytes of every table of a sweep (T_0 .. T_n), for tg_dense_witness_small; -1 on a bad op stream
int64_t tg_dense_witness_bytes(const int64_t *ops, int64_t n, int eb) {
    if ((eb != 1 && eb != 2) || n < 0 || (n && !ops)) return -1;
    int64_t w = 0, tot = 1;
    for (int64_t k = 0; k < n; k++) {
        const int64_t code = ops[3 * k];
        w += code == 0 ? 1 : code == 2 ? -1 : 0;
        if (w < 0 || w > 30) return -1;
        tot += 1ll << w;
    }
    return tot * eb;
}

// The witness of a small plan in one launch (ops: HOST int64 [n][3] as tg_dense_plan): every table
// of the sweep is kept in `tables` (DEVICE, tg_dense_witness_bytes bytes), one block applies the
// ops and one thread walks back.  out_dev: DEVICE int32 [3 + out_cap] = final entry, number of used
// updates, their op indices (last op first), then a status (0 ok, 1 bad op stream or storage, 2
// the walk lost the path).
int tg_dense_witness_small(const int64_t *ops, int64_t n, int eb, void *tables, uint64_t table_bytes,
                           int32_t *out_dev, int64_t out_cap, void *stream) {
    if ((eb != 1 && eb != 2) || n < 0 || (n && !ops) || !tables || !out_dev || out_cap < 0)
        return set_error(TG_ERR_ARG, "bad witness arguments");
    const int64_t need = tg_dense_witness_bytes(ops, n, eb);
    if (need < 0) return set_error(TG_ERR_ARG, "bad op stream");
    if ((uint64_t)need > table_bytes) return set_error(TG_ERR_TOO_BIG, "witness tables larger than the buffer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    static thread_local int64_t *dops = nullptr;
    static thread_local int64_t dops_n = 0;
    if (dops_n < n) {
        if (dops) cudaFree(dops);
        dops = nullptr;
        dops_n = 0;
        if (cudaMalloc(&dops, 24 * (size_t)std::max<int64_t>(n, 1)) != cudaSuccess) {
            cudaGetLastError();
            return set_error(TG_ERR_NOMEM, "witness op stream");
        }
        dops_n = n;
    }
    int e = TG_OK;
    if (n) e = cuda_check(cudaMemcpyAsync(dops, ops, 24 * (size_t)n, cudaMemcpyHostToDevice, st), "witness ops");
    if (!e) e = cuda_check(cudaMemsetAsync(out_dev, 0, 4 * (size_t)(3 + out_cap), st), "witness out");
    if (e) return e;
    const uint64_t cap = (uint64_t)need / eb;
    if (eb == 1)
        k_witness_small<uint8_t><<<1, 1024, 0, st>>>(dops, n, static_cast<uint8_t *>(tables), cap, out_dev, out_cap);
    else
        k_witness_small<uint16_t><<<1, 1024, 0, st>>>(dops, n, static_cast<uint16_t *>(tables), cap, out_dev, out_cap);
    return cuda_check(cudaGetLastError(), "witness kernel");
}
}  // extern "C"
