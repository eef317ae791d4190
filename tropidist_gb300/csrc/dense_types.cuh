// Types and device bodies shared by the dense kernels (dense.cu) and the batched persistent kernel
// (batch.cu): the shared-memory update, the narrow-table sweep, the fused-pass parameters and the
// host-side schedule of a plan.
#pragma once
#include "tg_common.cuh"
#include "fused_u8.cuh"

#include <cstring>
#include <vector>

namespace tg {

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

// a whole run of ops on a table held in shared memory (smem_raw: 2 x 2^max_bits entries), all
// threads of the block; has_in: the input table is read from `in`, else the table starts as {0: 0}
template <typename E>
__device__ __forceinline__ void sweep_body(const SweepParams &P, const E *__restrict__ in, E *__restrict__ out,
                                           uint4 *smem_raw) {
    constexpr int CB = Entry<E>::CB;
    E *T = reinterpret_cast<E *>(smem_raw);
    E *S = T + (1u << P.max_bits);
    int bits = P.w_in;
    uint32_t n = 1u << bits;
    if (P.has_in) {
        for (uint32_t s = threadIdx.x; s < n; s += blockDim.x) T[s] = __ldcg(in + s);
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
    // uint8 register-group form of the same updates (k_fused_pass_u8)
    int use_groups, ngroups;
    int store_mode;                    // output chunk from: 0 one smem chunk, 1 two chunks without local
                                       // bit sel_low (< 4), 2 byte gathers through pat
    int sel_low;
    int nslow;                         // updates with in-chunk bits, applied in shared memory
    uint8_t slow_idx[FP_MAXU];
    GroupDesc groups[FP_MAXG];
    uint8_t ucode[FP_MAXU];
    uint8_t uw[FP_MAXU];
    // coset-streaming form of a one-group uint8 pass (k_stream_pass_u8): thread k of a tile takes
    // the coset of chunk c0 = deposit(k, kpos) | cfix and goes global -> registers -> global
    int stream;                        // 1: the streaming form applies
    int s_mode;                        // 0 one output chunk per tile chunk; 1 output chunks from the
                                       // chunk pairs (x, x + 1) without in-chunk bit s_bit
    int s_bit, s_both;                 // mode 1: both halves of s_bit stored (evicted row) or only s_tgt
    uint32_t s_tgt, s_w;               // mode 1: target (selected row) / output offset of the evicted row
    int nk;                            // coset-number bits: a tile has 2^nk cosets, a block 512 >> nk tiles
    uint8_t kpos[16];                  // local chunk bit receiving coset-number bit j
    uint32_t cfix;                     // chunk bits fixed in every coset (selected rows outside the span)
    uint32_t expm;                     // chunk bits of the rows expanded in the pass (their 1-half is INF)
    uint32_t selm, selb;               // chunk bits of the selected rows in the span, and their targets
    uint32_t kin[16], kout[16];        // input / output offsets of coset-number bit j
    uint32_t xin[8], xout[8];          // input / output offsets of the coset members sxoff[x]
    uint32_t fin, fout;                // input / output offsets of cfix
    // canonical form: coset member x is chunk c0 ^ sxoff[x], sxoff spanned by the chunk parts of
    // the first (up to 3) independent updates; member x is held with its entries permuted by
    // XOR with sshift[x] (the XOR of those updates' in-chunk masks selected by x), which turns
    // each of those updates into a plain pairing of members x and x ^ 2^j (weights s_cw); the
    // other updates keep a residual code (s_rcode, s_rw)
    uint32_t sxoff[8];
    uint32_t s_selu[8][2];             // unpack selectors (even / odd lanes) of member x
    uint32_t s_selp[8];                // pack selector of member x
    uint8_t s_wsw[8];                  // word-index XOR of member x (bits 2..3 of sshift[x])
    uint8_t sshift[8];
    int s_nc, s_nres;
    int s_ws;                          // 1: some member is word-permuted (s_wsw)
    int s_pb;                          // mode 1: x bit of the member pairs (chunk bit 0)
    // lane dimension: a fourth coset dimension split across the lane pair (l, l ^ 16): the thread
    // with coset-number bit 4 set holds the coset shifted by s_lvec; the update along it exchanges
    // registers with __shfl_xor (code s_lcode: register xor | lane swap << 6, weight s_lw)
    int s_lane, nkt;                   // nkt = nk + s_lane: coset-number bits of a tile
    int s_lgen;                        // 1: the lane update has an in-chunk part (general path)
    int s_l2;                          // 1: input and output fit L2 together (stores stay cached)
    uint32_t s_lvec, s_lin, s_lout;
    uint8_t s_lcode, s_lw;
    uint8_t s_cw[4];
    uint8_t s_rcode[FP_MAXU], s_rw[FP_MAXU];
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

#define FP_THREADS 512
#define FP_TBITS 9

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
    int w_start = 0;        // width of the start table (0: {0: 0}; else given in buffer a, canonical)
    int final_w = 0;        // width of the final table (canonical order)
    int64_t n_updates;
    double pass_bytes;      // algorithmic bytes moved by the fused passes
    std::vector<float> seg_ms;  // per-segment launch time of the last timed execution
    double sweep_bytes;     // bytes read + written by the shared-memory sweeps
};


// Output chunk of a uint8 tile whose compacted entry 0 is tile entry sidx (the selected bits
// already in place): mode 0 one slot, 1 two slots without local bit sel_low (< 4), 2 byte gathers
// through pat; sm is the slot swizzle of the tile (tslot).
static __device__ __forceinline__ uint4 u8_out_chunk(const uint4 *TC, int mode, uint32_t sidx, const PassParams &P,
                                                    uint32_t sm) {
    constexpr int CB = 4;
    if (mode == 0) return TC[tslot(sidx >> CB, sm)];
    if (mode == 1) {
        const uint32_t s0 = tslot((sidx >> 5) << 1, sm);
        return gather_one_select(TC[s0], TC[s0 ^ 1u], P.sel_low, (sidx >> P.sel_low) & 1u);
    }
    const uint8_t *T = reinterpret_cast<const uint8_t *>(TC);
    uint32_t wd[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        uint32_t word = 0;
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const uint32_t b = sidx + P.pat[4 * k + e];
            word |= (uint32_t)T[(tslot(b >> CB, sm) << CB) | (b & 15u)] << (8 * e);
        }
        wd[k] = word;
    }
    return make_uint4(wd[0], wd[1], wd[2], wd[3]);
}

// One tile of a fused uint8 pass by one block of NT threads, without pipelining (the batched
// kernel's unit of work): load the tile's input chunks (cp.async, through L2), INF over the rows
// expanded in the pass, the register groups and the shared-memory updates, and the store of the
// selected halves in the output order.  TC: 2^d entries of shared memory.
template <int NT>
static __device__ void u8_tile(const PassParams &P, uint64_t tile, const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                        uint4 *TC) {
    constexpr int CB = 4;
    const uint32_t tid = threadIdx.x;
    const int nb_in = P.d_in - CB, nb_out = P.d_out - CB;
    const uint32_t nch_in = 1u << nb_in, nch_all = 1u << (P.d - CB), nch_out = 1u << nb_out;
    uint64_t ib = 0, ob = 0;
    for (int k = 0; k < P.n_outer; k++)
        if ((tile >> k) & 1ull) { ib += P.outer_in[k]; ob += P.outer_out[k]; }
    const uint32_t sm = P.use_groups ? 7u : 0u;        // slot swizzle of the register-group form
    for (uint32_t c = tid; c < nch_in; c += NT) cp_async16(TC + tslot(c, sm), in + ib + pdep_w64(c, P.loc_in + CB, nb_in));
    for (uint32_t c = nch_in + tid; c < nch_all; c += NT) TC[tslot(c, sm)] = make_uint4(~0u, ~0u, ~0u, ~0u);
    cp_async_wait_all();
    __syncthreads();
    uint8_t *T = reinterpret_cast<uint8_t *>(TC);
    if (P.use_groups) {
        for (int g = 0; g < P.ngroups; g++) {
            run_group<NT>(TC, P.d, P.groups[g], P.ucode, P.uw);
            __syncthreads();
        }
    } else {
        for (int u = 0; u < P.nupd; u++) {
            smem_update<uint8_t>(T, P.d, P.upd_mask[u], P.upd_w[u]);
            __syncthreads();
        }
    }
    const int mode = P.use_groups ? P.store_mode : (P.fast_out ? 0 : 2);
    for (uint32_t q = tid; q < nch_out; q += NT) {
        const uint64_t off = ob + pdep_w64(q, P.cmp_out + CB, nb_out);
        const uint32_t sidx = pdep_w32(q, P.cmp_smem + CB, nb_out) + P.sel_bits;
        *reinterpret_cast<uint4 *>(out + off) = u8_out_chunk(TC, mode, sidx, P, sm);
    }
}

// The tiles [t0, t1) of a fused uint8 pass by one block of FP_THREADS threads: the tile loads go
// through a three-buffer cp.async ring (tiles t + 1 and t + 2 load while tile t is computed), the
// updates run in register-resident groups, the selected halves are stored in the output order.
// Chunk c of a tile is handled by thread c % 256 in iteration c / 256: its offsets are the
// thread's own part (computed once) plus an iteration part that is the same for every thread
// (tables in shared memory), and the tile bases advance by a carry table (tile t+1 differs from
// tile t in the bits up to the lowest zero bit of t).
#define FP_MAXIT 8
static __device__ __forceinline__ void u8_pass_range(const PassParams &P, uint64_t t0, uint64_t t1,
                                           const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                                           uint4 *smem_raw) {
    constexpr int CB = 4;
    __shared__ uint64_t s_in_hi[FP_MAXIT], s_out_hi[FP_MAXIT];
    __shared__ uint32_t s_sm_hi[FP_MAXIT];
    __shared__ int64_t s_cin[FP_MAXOUTER], s_cout[FP_MAXOUTER];
    const uint32_t tid = threadIdx.x;
    const int nb_in = P.d_in - CB, nb_out = P.d_out - CB;
    const int tb_in = min(nb_in, FP_TBITS), tb_out = min(nb_out, FP_TBITS);
    const uint32_t nch_in = 1u << nb_in, nch_all = 1u << (P.d - CB), nch_out = 1u << nb_out;
    const uint32_t it_in = (nch_in + FP_THREADS - 1) / FP_THREADS, it_out = (nch_out + FP_THREADS - 1) / FP_THREADS;
    if (tid < it_in) s_in_hi[tid] = pdep_w64(tid, P.loc_in + CB + FP_TBITS, nb_in - tb_in);
    if (tid < it_out) {
        s_out_hi[tid] = pdep_w64(tid, P.cmp_out + CB + FP_TBITS, nb_out - tb_out);
        s_sm_hi[tid] = pdep_w32(tid, P.cmp_smem + CB + FP_TBITS, nb_out - tb_out);
    }
    if (tid < (uint32_t)P.n_outer) {
        // carry table: base(t + 1) - base(t) when bit tid is the lowest zero bit of t
        int64_t ci = (int64_t)P.outer_in[tid], co = (int64_t)P.outer_out[tid];
        for (uint32_t k = 0; k < tid; k++) { ci -= (int64_t)P.outer_in[k]; co -= (int64_t)P.outer_out[k]; }
        s_cin[tid] = ci;
        s_cout[tid] = co;
    }
    const uint64_t tid_in = pdep_w64(tid, P.loc_in + CB, tb_in);
    const uint64_t tid_out = pdep_w64(tid, P.cmp_out + CB, tb_out);
    const uint32_t tid_sm = pdep_w32(tid, P.cmp_smem + CB, tb_out) + P.sel_bits;
    const bool in_full = nch_in >= FP_THREADS, out_full = nch_out >= FP_THREADS;

    uint64_t ib0 = 0, ob0 = 0;
    for (int k = 0; k < P.n_outer; k++)
        if ((t0 >> k) & 1ull) { ib0 += P.outer_in[k]; ob0 += P.outer_out[k]; }
    __syncthreads();

    const uint8_t *inb = in + tid_in;
    auto issue_load = [&](uint64_t ib, uint4 *TC) {
        const uint8_t *src = inb + ib;
        if (in_full) {
            for (uint32_t it = 0; it < it_in; it++) cp_async16(TC + tslot(it * FP_THREADS + tid, 7u), src + s_in_hi[it]);
        } else if (tid < nch_in) {
            cp_async16(TC + tslot(tid, 7u), src);
        }
        for (uint32_t c = nch_in + tid; c < nch_all; c += FP_THREADS) TC[tslot(c, 7u)] = make_uint4(~0u, ~0u, ~0u, ~0u);
        cp_async_commit();
    };
    auto advance = [&](uint64_t t, uint64_t &ib, uint64_t &ob) {   // bases of tile t + 1 from tile t
        const int k = __ffsll((long long)~t) - 1;
        ib += s_cin[k];
        ob += s_cout[k];
    };

    // three tile buffers: tiles t + 1 and t + 2 load while tile t is computed and stored
    uint4 *const buf0 = smem_raw, *const buf1 = smem_raw + nch_all, *const buf2 = smem_raw + 2 * nch_all;
    int cur = 0;
    uint64_t ob = ob0, ibn = ib0, dummy = 0;
    uint64_t tl = t0;          // next tile to load (ibn: its input base)
    if (tl < t1) { issue_load(ibn, buf0); tl++; }
    if (tl < t1) { advance(tl - 1, ibn, dummy); issue_load(ibn, buf1); tl++; }
    for (uint64_t tile = t0; tile < t1; tile++) {
        if (tl < t1) {
            advance(tl - 1, ibn, dummy);
            const int slot = (cur + 2) % 3;
            issue_load(ibn, slot == 0 ? buf0 : slot == 1 ? buf1 : buf2);
            tl++;
        }
        const uint64_t ahead = tl - 1 - tile;        // loads still allowed in flight
        if (ahead >= 2) cp_async_wait_group<2>();
        else if (ahead == 1) cp_async_wait_group<1>();
        else cp_async_wait_group<0>();
        __syncthreads();
        uint4 *TC = cur == 0 ? buf0 : cur == 1 ? buf1 : buf2;
        for (int g = 0; g < P.ngroups; g++) {
            run_group<FP_THREADS>(TC, P.d, P.groups[g], P.ucode, P.uw);
            __syncthreads();
        }
        uint8_t *dstb = out + ob + tid_out;
        for (uint32_t it = 0; it < it_out; it++) {
            const uint32_t q = it * FP_THREADS + tid;
            if (!out_full && q >= nch_out) break;
            const uint32_t sidx = tid_sm + s_sm_hi[it];
            __stcs(reinterpret_cast<uint4 *>(dstb + s_out_hi[it]), u8_out_chunk(TC, P.store_mode, sidx, P, 7u));
        }
        __syncthreads();
        cur = cur == 2 ? 0 : cur + 1;
        if (tile + 1 < t1) advance(tile, dummy, ob);
    }
}


// ------------------------------------------------------------------ coset-streaming pass (uint8)
// the update along the lane dimension: register I takes min(R[I], partner lane's R[I ^ X] + w)
// (lanes swapped when HS); pairs (I, I ^ X) read both partner values before writing
template <int X, int HS, int I>
struct LanePairs {
    static __device__ __forceinline__ void run(uint32_t (&R)[64], uint32_t w2) {
        if constexpr (X == 0) {
            uint32_t v = __shfl_xor_sync(0xFFFFFFFFu, R[I], 16);
            if constexpr (HS) v = swap_halves(v);
            R[I] = __viaddmin_u16x2(v, w2, R[I]);
        } else if constexpr (I < (I ^ X)) {
            uint32_t a = __shfl_xor_sync(0xFFFFFFFFu, R[I ^ X], 16), b = __shfl_xor_sync(0xFFFFFFFFu, R[I], 16);
            if constexpr (HS) { a = swap_halves(a); b = swap_halves(b); }
            R[I] = __viaddmin_u16x2(a, w2, R[I]);
            R[I ^ X] = __viaddmin_u16x2(b, w2, R[I ^ X]);
        }
        if constexpr (I < 63) LanePairs<X, HS, I + 1>::run(R, w2);
    }
};

// code: register xor (bits 0..2: word and parity of the in-chunk part) | lane swap << 6
static __device__ __forceinline__ void lane_dispatch(uint32_t code, uint32_t (&R)[64], uint32_t w2) {
    switch (code) {
        case 0: LanePairs<0, 0, 0>::run(R, w2); break;
        case 1: LanePairs<1, 0, 0>::run(R, w2); break;
        case 2: LanePairs<2, 0, 0>::run(R, w2); break;
        case 3: LanePairs<3, 0, 0>::run(R, w2); break;
        case 4: LanePairs<4, 0, 0>::run(R, w2); break;
        case 5: LanePairs<5, 0, 0>::run(R, w2); break;
        case 6: LanePairs<6, 0, 0>::run(R, w2); break;
        case 7: LanePairs<7, 0, 0>::run(R, w2); break;
        case 64: LanePairs<0, 1, 0>::run(R, w2); break;
        case 65: LanePairs<1, 1, 0>::run(R, w2); break;
        case 66: LanePairs<2, 1, 0>::run(R, w2); break;
        case 67: LanePairs<3, 1, 0>::run(R, w2); break;
        case 68: LanePairs<4, 1, 0>::run(R, w2); break;
        case 69: LanePairs<5, 1, 0>::run(R, w2); break;
        case 70: LanePairs<6, 1, 0>::run(R, w2); break;
        case 71: LanePairs<7, 1, 0>::run(R, w2); break;
        default: break;
    }
}

// ---- the coset of one thread in one step (straight-line code, no per-member switches)
// member x's 16 entries widened into R[8x .. 8x + 7] (u16 lanes) in the canonical permuted form: the
// unpack selectors realise the in-chunk XOR on entry bits 0-1, and for word-permuted members (WS)
// the entry word k is read from storage word k ^ wsw (bits 2-3) by its shared-memory address
template <bool WS>
static __device__ __forceinline__ void u8_unpack_member(const PassParams &P, const uint8_t *src, int x, bool is_inf,
                                                        uint32_t *R) {
    uint32_t w0, w1, w2, w3;
    if (WS) {
        const uint32_t ws4 = 4u * P.s_wsw[x];
        const uint8_t *m = src + x * 512;
        w0 = *reinterpret_cast<const uint32_t *>(m + (0u ^ ws4));
        w1 = *reinterpret_cast<const uint32_t *>(m + (4u ^ ws4));
        w2 = *reinterpret_cast<const uint32_t *>(m + (8u ^ ws4));
        w3 = *reinterpret_cast<const uint32_t *>(m + (12u ^ ws4));
    } else {
        const uint4 v = *reinterpret_cast<const uint4 *>(src + x * 512);
        w0 = v.x; w1 = v.y; w2 = v.z; w3 = v.w;
    }
    if (is_inf) w0 = w1 = w2 = w3 = 0xFFFFFFFFu;
    const uint32_t se = P.s_selu[x][0], so = P.s_selu[x][1];
    R[0] = __byte_perm(w0, 0u, se); R[1] = __byte_perm(w0, 0u, so);
    R[2] = __byte_perm(w1, 0u, se); R[3] = __byte_perm(w1, 0u, so);
    R[4] = __byte_perm(w2, 0u, se); R[5] = __byte_perm(w2, 0u, so);
    R[6] = __byte_perm(w3, 0u, se); R[7] = __byte_perm(w3, 0u, so);
}

// member x back to its 16 bytes in storage order
template <bool WS>
static __device__ __forceinline__ uint4 u8_pack_member(const PassParams &P, int x, const uint32_t *R) {
    const uint32_t sp = P.s_selp[x];
    const uint32_t q0 = __byte_perm(R[0], R[1], sp), q1 = __byte_perm(R[2], R[3], sp);
    const uint32_t q2 = __byte_perm(R[4], R[5], sp), q3 = __byte_perm(R[6], R[7], sp);
    if (!WS) return make_uint4(q0, q1, q2, q3);
    // storage word k holds entry word k ^ wsw
    const uint32_t ws = P.s_wsw[x];
    const bool b0 = ws & 1u, b1 = ws & 2u;
    const uint32_t t0 = b0 ? q1 : q0, t1 = b0 ? q0 : q1, t2 = b0 ? q3 : q2, t3 = b0 ? q2 : q3;
    return b1 ? make_uint4(t2, t3, t0, t1) : make_uint4(t0, t1, t2, t3);
}

// the coset's updates on its registers: NC canonical member pairings, the lane update, or (GEN) every
// update through its code
template <int NC, bool GEN>
static __device__ __forceinline__ void u8_stream_updates(const PassParams &P, uint32_t (&R)[64]) {
    if constexpr (GEN) {
        for (int u = 0; u < P.s_nc; u++) {
            const uint32_t w = P.s_cw[u];
            reg_dispatch(8u << u, R, w | (w << 16));
        }
        for (int u = 0; u < P.s_nres; u++) {
            const uint32_t w = P.s_rw[u];
            reg_dispatch(P.s_rcode[u], R, w | (w << 16));
        }
    }
    if constexpr (!GEN && NC >= 1) { const uint32_t w = P.s_cw[0]; RegPairs<8, 0, 0>::run(R, w | (w << 16)); }
    if constexpr (!GEN && NC >= 2) { const uint32_t w = P.s_cw[1]; RegPairs<16, 0, 0>::run(R, w | (w << 16)); }
    if constexpr (!GEN && NC >= 3) { const uint32_t w = P.s_cw[2]; RegPairs<32, 0, 0>::run(R, w | (w << 16)); }
    if (P.s_lane) {                    // uniform: every lane of the warp takes this branch
        const uint32_t w = P.s_lw;
        if (GEN) lane_dispatch(P.s_lcode, R, w | (w << 16));
        else LanePairs<0, 0, 0>::run(R, w | (w << 16));
    }
}

// an output chunk: kept in L2 when the next pass reads it from there, else streamed out
static __device__ __forceinline__ void u8_store(const PassParams &P, uint8_t *p, const uint4 &v) {
    if (P.s_l2) __stcg(reinterpret_cast<uint4 *>(p), v);
    else __stcs(reinterpret_cast<uint4 *>(p), v);
}

// mode-1 output chunks: the member pairs (x, x ^ PB) that differ in chunk bit 0, without in-chunk
// bit s_bit (one or both halves stored)
template <int PB, bool WS>
static __device__ __forceinline__ void u8_stream_store_pairs(const PassParams &P, const uint32_t (&R)[64],
                                                            uint32_t keep, uint8_t *dst, uint32_t outc, uint32_t c0b) {
#pragma unroll
    for (int x = 0; x < 8; x++) {
        if (x & PB) continue;
        if (!((keep >> x) & 1u)) continue;
        const uint4 M0 = u8_pack_member<WS>(P, x, R + 8 * x), M1 = u8_pack_member<WS>(P, x | PB, R + 8 * (x | PB));
        const bool sw = (P.sxoff[x] ^ c0b) & 1u;   // member x has chunk bit 0 set: it is the upper one
        const uint4 A = sw ? M1 : M0, B = sw ? M0 : M1;
        uint8_t *const o = dst + (outc ^ P.xout[x]);
        if (P.s_both) {
            u8_store(P, o, gather_one_select(A, B, P.s_bit, 0u));
            u8_store(P, o + P.s_w, gather_one_select(A, B, P.s_bit, 1u));
        } else {
            u8_store(P, o, gather_one_select(A, B, P.s_bit, P.s_tgt));
        }
    }
}

// A one-group pass without a shared-memory tile: thread k of tile t owns the coset {c0 ^ X[x]} of
// the tile's chunks (c0 fixed per thread for the whole launch), stages its 8 input chunks in its
// own shared-memory slots with cp.async three tiles ahead (no barriers: a thread reads back only
// its own copies), applies the group's updates in registers and stores the output chunks straight
// to global memory, member by member.  A block covers 512 >> nk tiles per step; steps [s0, s1) in
// order.  The variant (canonical updates, word permutation, general codes) is chosen once per range.
#define FS_STAGES 3
#define FS_WARP_BYTES (FS_STAGES * 8 * 512)      // staging bytes of one warp

template <int NC, bool WS, bool GEN>
static __device__ __forceinline__ void u8_stream_loop(const PassParams &P, uint64_t s0, uint64_t s1,
                                                      const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                                                      uint8_t *stage0, const int64_t *s_cin, const int64_t *s_cout,
                                                      int g, int ng, uint32_t j, uint32_t keep, uint32_t inf,
                                                      uint32_t c0b, uint32_t inc, uint32_t outc, uint64_t ib,
                                                      uint64_t ob) {
    const uint64_t ntiles = P.ntiles;
    auto issue = [&](uint64_t s, uint64_t b, int st) {
        if ((((s << g) | j) < ntiles)) {
            uint8_t *dst = stage0 + st * 4096;
            const uint8_t *base = in + b;
#pragma unroll
            for (int x = 0; x < 8; x++)
                if (!((inf >> x) & 1u)) cp_async16(dst + x * 512, base + (inc ^ P.xin[x]));
        }
        cp_async_commit();
    };
    auto advance = [&](uint64_t s, uint64_t &bi, uint64_t &bo) {   // bases of step s + 1 from step s
        const int q = __ffsll((long long)~s) - 1 + ng;
        if (q < P.n_outer) { bi += s_cin[q]; bo += s_cout[q]; }
    };
    uint64_t ibn = ib, dummy = 0;
    // prologue: steps s0 and s0 + 1 in flight
    issue(s0, ibn, 0);
    if (s0 + 1 < s1) {
        advance(s0, ibn, dummy);
        issue(s0 + 1, ibn, 1);
    } else {
        cp_async_commit();
    }
    int st = 0;
    for (uint64_t s = s0; s < s1; s++) {
        if (s + 2 < s1) {
            advance(s + 1, ibn, dummy);
            issue(s + 2, ibn, st == 0 ? 2 : st - 1);
        } else {
            cp_async_commit();
        }
        cp_async_wait_group<2>();
        if (((s << g) | j) < ntiles) {
            const uint8_t *src = stage0 + st * 4096;
            uint32_t R[64];
#pragma unroll
            for (int x = 0; x < 8; x++) u8_unpack_member<WS>(P, src, x, (inf >> x) & 1u, R + 8 * x);
            u8_stream_updates<NC, GEN>(P, R);
            uint8_t *const dst = out + ob;
            if (P.s_mode == 0) {
#pragma unroll
                for (int x = 0; x < 8; x++)
                    if ((keep >> x) & 1u) u8_store(P, dst + (outc ^ P.xout[x]), u8_pack_member<WS>(P, x, R + 8 * x));
            } else if (P.s_pb == 0) {
                u8_stream_store_pairs<1, WS>(P, R, keep, dst, outc, c0b);
            } else if (P.s_pb == 1) {
                u8_stream_store_pairs<2, WS>(P, R, keep, dst, outc, c0b);
            } else {
                u8_stream_store_pairs<4, WS>(P, R, keep, dst, outc, c0b);
            }
        }
        st = st == FS_STAGES - 1 ? 0 : st + 1;
        if (s + 1 < s1) advance(s, dummy, ob);
    }
    cp_async_wait_group<0>();
}

static __device__ __forceinline__ void u8_stream_range(const PassParams &P, uint64_t s0, uint64_t s1,
                                                   const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                                                   uint4 *smem_raw) {
    __shared__ int64_t s_cin[FP_MAXOUTER], s_cout[FP_MAXOUTER];
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const int g = 9 - P.nkt;                           // log2 of the tiles per step
    const uint32_t k = tid & ((1u << P.nkt) - 1u), j = tid >> P.nkt;
    const int ng = min(g, P.n_outer);
    if (tid < (uint32_t)P.n_outer && (int)tid >= ng) {
        // carry table of the step index: base(s + 1) - base(s) when bit tid - ng is the lowest zero bit of s
        int64_t ci = (int64_t)P.outer_in[tid], co = (int64_t)P.outer_out[tid];
        for (int q = ng; q < (int)tid; q++) { ci -= (int64_t)P.outer_in[q]; co -= (int64_t)P.outer_out[q]; }
        s_cin[tid] = ci;
        s_cout[tid] = co;
    }
    // the thread's coset (constant for the launch): its chunk offsets, kept and INF members
    uint32_t c0 = P.cfix, inc = P.fin, outc = P.fout;
    for (int q = 0; q < P.nk; q++) {
        const int bit = (P.s_lane && q >= 4) ? q + 1 : q;      // bit 4 is the lane dimension
        if ((k >> bit) & 1u) { c0 ^= 1u << P.kpos[q]; inc ^= P.kin[q]; outc ^= P.kout[q]; }
    }
    if (P.s_lane && ((k >> 4) & 1u)) { c0 ^= P.s_lvec; inc ^= P.s_lin; outc ^= P.s_lout; }
    uint32_t keep = 0, inf = 0;
#pragma unroll
    for (int x = 0; x < 8; x++) {
        const uint32_t c = c0 ^ P.sxoff[x];
        if ((c & P.selm) == P.selb) keep |= 1u << x;
        if (c & P.expm) inf |= 1u << x;
    }
    uint64_t jin = 0, jout = 0;                        // the thread's tile within a step
    for (int q = 0; q < ng; q++)
        if ((j >> q) & 1u) { jin += P.outer_in[q]; jout += P.outer_out[q]; }
    uint64_t ib = jin, ob = jout;                      // bases of step s0
    for (int q = ng; q < P.n_outer; q++)
        if ((s0 >> (q - ng)) & 1ull) { ib += P.outer_in[q]; ob += P.outer_out[q]; }
    __syncthreads();
    // programmatic dependent launch: everything above overlapped the previous pass; its writes (our
    // input) and reads (our output buffer) are complete past this point
    asm volatile("griddepcontrol.wait;" ::: "memory");

    uint8_t *const stage0 = reinterpret_cast<uint8_t *>(smem_raw) + (size_t)warp * FS_WARP_BYTES + lane * 16u;
    const uint32_t c0b = c0 & 1u;
#define TG_SLOOP(NC, WS, GEN) \
    u8_stream_loop<NC, WS, GEN>(P, s0, s1, in, out, stage0, s_cin, s_cout, g, ng, j, keep, inf, c0b, inc, outc, ib, ob)
    if (P.s_nres || P.s_lgen) {
        TG_SLOOP(0, true, true);
    } else {
        switch (P.s_nc + 4 * P.s_ws) {
            case 0: TG_SLOOP(0, false, false); break;
            case 1: TG_SLOOP(1, false, false); break;
            case 2: TG_SLOOP(2, false, false); break;
            case 3: TG_SLOOP(3, false, false); break;
            case 4: TG_SLOOP(0, true, false); break;
            case 5: TG_SLOOP(1, true, false); break;
            case 6: TG_SLOOP(2, true, false); break;
            default: TG_SLOOP(3, true, false); break;
        }
    }
#undef TG_SLOOP
}

// on_seg (optional): called with every segment as soon as it is scheduled (a nonzero return stops
// the scheduler with that status), so that the caller can launch it before the rest is scheduled
using SegHook = int (*)(const Seg &S, void *ctx);
int build_dense_plan(const int64_t *ops, int64_t nops, int eb, const int64_t *ckpts, int64_t nckpt, DensePlan &P,
                     int w_start = 0, bool open_end = false, SegHook on_seg = nullptr, void *hook_ctx = nullptr);
int set_dense_attrs();

}  // namespace tg
