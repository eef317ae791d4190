// Batched dense Rank DP: many independent plans (the logical observables of many instances) run in
// one persistent launch fed from a device work queue.
//
// Each plan is scheduled as in dense.cu (shared-memory sweeps, fused passes, one-op passes); every
// segment of every plan becomes a job of one or more units: a sweep is one unit (one block runs it
// in shared memory), a fused pass has one unit per tile, a one-op pass one unit per 4096 chunks.
// A plan's segments must run in order, different plans are independent, so:
//   - the queue starts with the first job of every plan;
//   - a block takes a unit of the job at the queue head (an atomic counter per job) and advances the
//     head when the job's units are exhausted;
//   - the block that completes a job's last unit appends the plan's next job to the queue (its
//     writes, and every block's writes of that job, are fenced before the completion count);
//   - blocks that find no job poll with a bounded number of iterations, then set an error flag and
//     return (status TG_ERR_TIMEOUT on the host): no wait is unbounded.
// Each plan's two tables live in a caller-provided arena (a per-instance frontier arena).
#include "tg_common.cuh"
#include "tg_capi.h"
#include "dense_types.cuh"

#include <algorithm>
#include <cstring>
#include <vector>

namespace tg {

#define BJ_NONE 0xFFFFFFFFu
#define BJ_UNIT_CHUNKS 4096u
#define BT_THREADS FP_THREADS

struct BJob {
    int kind;                // 0 sweep, 1 fused pass, 2 one-op pass
    int plan;
    uint32_t nunits;
    uint32_t next;           // the plan's next job (BJ_NONE: the plan ends)
    uint64_t params_off;     // SweepParams / PassParams in the parameter blob
    uint64_t src_off, dst_off;
    int bits;                // one-op pass: width of the input table
    int op_code;
    uint64_t op_a;
    uint32_t op_b;
    uint32_t grain;          // fused pass: tiles per unit
};

struct BatchArgs {
    const BJob *jobs;
    const uint8_t *params;
    uint8_t *arena;
    unsigned *taken, *done, *queue, *ready;
    unsigned *ctl;           // head, tail, finished plans, error flags, next plan to admit
    const unsigned *admit;   // plans' first jobs in admission order
    unsigned nadmit;         // plans in the admission list
    unsigned nplans;
    unsigned long long spin_limit;
};

__device__ __forceinline__ unsigned ld_volatile(const unsigned *p) { return *(volatile const unsigned *)p; }

// thread 0: the next unit; state 0 job, 1 all plans finished, 2 wait limit reached
__device__ void batch_grab(const BatchArgs &A, int &state, unsigned &job, unsigned &unit) {
    for (unsigned long long it = 0; it < A.spin_limit; it++) {
        if (ld_volatile(A.ctl + 2) >= A.nplans) { state = 1; return; }
        const unsigned h = ld_volatile(A.ctl + 0), t = ld_volatile(A.ctl + 1);
        if (h < t) {
            if (!ld_volatile(A.ready + h)) { __nanosleep(64); continue; }
            __threadfence();
            const unsigned j = ld_volatile(A.queue + h);
            const unsigned u = atomicAdd(A.taken + j, 1u);
            if (u < A.jobs[j].nunits) { state = 0; job = j; unit = u; __threadfence(); return; }
            atomicCAS(A.ctl + 0, h, h + 1);
            continue;
        }
        __nanosleep(128);
    }
    atomicOr(A.ctl + 3, 1u);
    state = 2;
}

__device__ void batch_single_op(const BJob &J, unsigned unit, const uint8_t *src, uint8_t *dst) {
    const uint64_t n = 1ull << J.bits;
    const uint64_t c0 = (uint64_t)unit * BJ_UNIT_CHUNKS, c1 = c0 + BJ_UNIT_CHUNKS;
    const Chunk *S = reinterpret_cast<const Chunk *>(src);
    Chunk *D = reinterpret_cast<Chunk *>(dst);
    if (J.op_code == 1) {
        const uint64_t hhi = J.op_a >> 4;
        const uint32_t hlo = (uint32_t)(J.op_a & 15u);
        for (uint64_t c = c0 + threadIdx.x; c < c1 && c < (n >> 4); c += blockDim.x) {
            Chunk a = ld_chunk_cg(S + c), b = chunk_xor<uint8_t>(ld_chunk_cg(S + (c ^ hhi)), hlo);
            st_chunk(D + c, chunk_minplus<uint8_t>(a, b, J.op_b));
        }
    } else if (J.op_code == 0) {
        Chunk inf;
        inf.w[0] = inf.w[1] = inf.w[2] = inf.w[3] = 0xFFFFFFFFu;
        for (uint64_t c = c0 + threadIdx.x; c < c1 && c < (n >> 4); c += blockDim.x) {
            st_chunk(D + c, ld_chunk_cg(S + c));
            st_chunk(D + (n >> 4) + c, inf);
        }
    } else {
        const int pos = (int)J.op_a;
        if (pos >= 4) {
            for (uint64_t q = c0 + threadIdx.x; q < c1 && q < (n >> 5); q += blockDim.x)
                st_chunk(D + q, ld_chunk_cg(S + (insert_zero64(q, pos - 4) | ((uint64_t)J.op_b << (pos - 4)))));
        } else {
            for (uint64_t k = c0 * 16 + threadIdx.x; k < c1 * 16 && k < (n >> 1); k += blockDim.x)
                dst[k] = __ldcg(src + (insert_zero64(k, pos) | ((uint64_t)J.op_b << pos)));
        }
    }
}

#define BT_TILE_SMEM (3 * 65536)
__global__ void __launch_bounds__(BT_THREADS, 1) k_batch(const __grid_constant__ BatchArgs A) {
    extern __shared__ uint4 smem_raw[];
    // layout: three 64 KB tile buffers (a sweep uses the first two), then the job's parameters
    uint4 *TC = smem_raw;
    uint4 *PRM = smem_raw + (BT_TILE_SMEM / 16);
    __shared__ int s_state;
    __shared__ unsigned s_job, s_unit;
    for (;;) {
        if (threadIdx.x == 0) {
            int st;
            unsigned j = 0, u = 0;
            batch_grab(A, st, j, u);
            s_state = st;
            s_job = j;
            s_unit = u;
        }
        __syncthreads();
        if (s_state != 0) break;
        const BJob J = A.jobs[s_job];
        const unsigned unit = s_unit;
        const uint8_t *src = A.arena + J.src_off;
        uint8_t *dst = A.arena + J.dst_off;
        if (J.kind == 0 || J.kind == 1) {
            const size_t psize = J.kind == 0 ? sizeof(SweepParams) : sizeof(PassParams);
            const uint4 *g = reinterpret_cast<const uint4 *>(A.params + J.params_off);
            for (uint32_t i = threadIdx.x; i < (psize + 15) / 16; i += blockDim.x) PRM[i] = g[i];
            __syncthreads();
            if (J.kind == 0) {
                sweep_body<uint8_t>(*reinterpret_cast<const SweepParams *>(PRM), src, dst, TC);
            } else {
                const PassParams &P = *reinterpret_cast<const PassParams *>(PRM);
                const uint64_t t0 = (uint64_t)unit * J.grain;
                const uint64_t t1 = t0 + J.grain < P.ntiles ? t0 + J.grain : P.ntiles;
                if (P.use_groups) u8_pass_range(P, t0, t1, src, dst, TC);
                else
                    for (uint64_t t = t0; t < t1; t++) {
                        u8_tile<BT_THREADS>(P, t, src, dst, TC);
                        __syncthreads();
                    }
            }
        } else {
            batch_single_op(J, unit, src, dst);
        }
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            const unsigned prev = atomicAdd(A.done + s_job, 1u);
            if (prev + 1 == J.nunits) {
                if (J.next != BJ_NONE) {
                    const unsigned slot = atomicAdd(A.ctl + 1, 1u);
                    A.queue[slot] = J.next;
                    __threadfence();
                    atomicExch(A.ready + slot, 1u);
                } else {
                    // the plan is done: admit the next waiting plan, then count this one
                    const unsigned k = atomicAdd(A.ctl + 4, 1u);
                    if (k < A.nadmit) {
                        const unsigned slot = atomicAdd(A.ctl + 1, 1u);
                        A.queue[slot] = A.admit[k];
                        __threadfence();
                        atomicExch(A.ready + slot, 1u);
                    }
                    __threadfence();
                    atomicAdd(A.ctl + 2, 1u);
                }
            }
        }
        __syncthreads();
    }
}

struct BatchPlan {
    int nplans = 0;
    std::vector<BJob> jobs;
    std::vector<uint8_t> params;
    std::vector<unsigned> first;         // first job per plan (BJ_NONE: empty plan)
    std::vector<uint64_t> final_off;     // arena offset of each plan's final table
    std::vector<int> width;              // peak width of each plan
    uint64_t arena_bytes = 0;
    int64_t units = 0;
    void *dev = nullptr;                 // jobs, params, counters
    size_t dev_bytes = 0;
    size_t off_jobs = 0, off_params = 0, off_cnt = 0, off_vals = 0, off_offs = 0;
    unsigned ncnt = 0;
};

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

static_assert(sizeof(SweepParams) <= 4096 && sizeof(PassParams) <= 4096, "job parameters exceed their 4 KB copy");

static bool g_batch_attr = false;

}  // namespace tg

using namespace tg;

extern "C" {

// Schedules nplans plans (op streams ops[offsets[i] .. offsets[i+1]) rows of int64 (code, a, b),
// uint8 tables) into one batch.  NULL and *status on failure.
void *tg_batch_create(int nplans, const int64_t *ops, const int64_t *offsets, int *status) {
    int st = TG_OK;
    BatchPlan *B = nullptr;
    if (nplans <= 0 || !offsets || !ops) st = set_error(TG_ERR_ARG, "bad batch");
    if (!st) {
        B = new BatchPlan();
        B->nplans = nplans;
        B->first.assign(nplans, BJ_NONE);
        B->final_off.assign(nplans, 0);
        B->width.assign(nplans, 0);
        for (int i = 0; i < nplans && !st; i++) {
            const int64_t n = offsets[i + 1] - offsets[i];
            if (n < 0) { st = set_error(TG_ERR_ARG, "bad plan offsets"); break; }
            DensePlan P;
            st = build_dense_plan(ops + 3 * offsets[i], n, 1, nullptr, 0, P);
            if (st) break;
            for (const Seg &S : P.segs)
                if ((S.kind == 0 && S.sp.max_bits > 15) || (S.kind == 1 && S.pp.d > 16)) {
                    st = set_error(TG_ERR_TOO_BIG, "batched plans need sweeps of <= 15 bits and tiles of <= 16 bits");
                    break;
                }
            if (st) break;
            B->width[i] = P.peak_bits;
            const uint64_t tb = align_up((size_t)1 << P.peak_bits, 256);
            const uint64_t a = B->arena_bytes, b = a + tb;
            B->arena_bytes = b + tb;
            B->final_off[i] = P.final_buf ? b : a;
            int cur = 0;
            unsigned prev = BJ_NONE;
            for (const Seg &S : P.segs) {
                BJob J;
                memset(&J, 0, sizeof(J));
                J.plan = i;
                J.next = BJ_NONE;
                J.src_off = cur ? b : a;
                J.dst_off = cur ? a : b;
                if (S.kind == 0) {
                    J.kind = 0;
                    J.nunits = 1;
                    J.params_off = align_up(B->params.size(), 16);
                    B->params.resize(J.params_off + sizeof(SweepParams));
                    memcpy(B->params.data() + J.params_off, &S.sp, sizeof(SweepParams));
                } else if (S.kind == 1) {
                    J.kind = 1;
                    const uint64_t nt = S.pp.ntiles;
                    // large units amortise the per-unit overhead; concurrency comes from the other plans
                    J.grain = (uint32_t)std::min<uint64_t>(nt, std::max<uint64_t>(16, (nt + sm_count() - 1) / sm_count()));
                    J.nunits = (uint32_t)((nt + J.grain - 1) / J.grain);
                    J.params_off = align_up(B->params.size(), 16);
                    B->params.resize(J.params_off + sizeof(PassParams));
                    memcpy(B->params.data() + J.params_off, &S.pp, sizeof(PassParams));
                } else {
                    J.kind = 2;
                    J.bits = S.w_in;
                    J.op_code = S.op_code;
                    J.op_a = S.op_a;
                    J.op_b = S.op_b;
                    const uint64_t chunks = std::max<uint64_t>(1, ((uint64_t)1 << S.w_in) >> 4);
                    J.nunits = (uint32_t)((chunks + BJ_UNIT_CHUNKS - 1) / BJ_UNIT_CHUNKS);
                }
                B->units += J.nunits;
                const unsigned idx = (unsigned)B->jobs.size();
                if (prev == BJ_NONE) B->first[i] = idx;
                else B->jobs[prev].next = idx;
                B->jobs.push_back(J);
                prev = idx;
                cur ^= 1;
            }
        }
        if (!st) {
            const size_t nj = std::max<size_t>(1, B->jobs.size());
            B->ncnt = (unsigned)(4 * nj + 8 + nplans);
            B->off_jobs = 0;
            B->off_params = align_up(nj * sizeof(BJob), 256);
            B->off_cnt = align_up(B->off_params + std::max<size_t>(16, B->params.size()), 256);
            B->off_vals = align_up(B->off_cnt + (size_t)B->ncnt * 4, 256);
            B->off_offs = align_up(B->off_vals + (size_t)nplans, 256);
            B->dev_bytes = B->off_offs + (size_t)nplans * 8;
            if (cudaMalloc(&B->dev, B->dev_bytes) != cudaSuccess) {
                cudaGetLastError();
                st = set_error(TG_ERR_NOMEM, "batch descriptors");
            } else {
                uint8_t *d = static_cast<uint8_t *>(B->dev);
                if (!B->jobs.empty())
                    st = cuda_check(cudaMemcpy(d + B->off_jobs, B->jobs.data(), B->jobs.size() * sizeof(BJob),
                                               cudaMemcpyHostToDevice), "batch jobs");
                if (!st && !B->params.empty())
                    st = cuda_check(cudaMemcpy(d + B->off_params, B->params.data(), B->params.size(),
                                               cudaMemcpyHostToDevice), "batch params");
                if (!st)
                    st = cuda_check(cudaMemcpy(d + B->off_offs, B->final_off.data(), (size_t)nplans * 8,
                                               cudaMemcpyHostToDevice), "batch offsets");
            }
        }
        if (st) {
            if (B->dev) cudaFree(B->dev);
            delete B;
            B = nullptr;
        }
    }
    if (status) *status = st;
    return B;
}

// Bytes of device memory the caller's arena must provide; units of work in the batch.
int tg_batch_info(void *p, int64_t *info, int ninfo) {
    if (!p || !info) return set_error(TG_ERR_ARG, "null batch");
    const BatchPlan &B = *static_cast<BatchPlan *>(p);
    int64_t v[4] = {(int64_t)B.arena_bytes, (int64_t)B.jobs.size(), B.units, B.nplans};
    for (int k = 0; k < ninfo && k < 4; k++) info[k] = v[k];
    return TG_OK;
}

__global__ void k_batch_values(const uint8_t *arena, const uint64_t *offs, int n, uint8_t *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = arena[offs[i]];
}

// Runs the batch in one persistent launch on `arena` (device, >= arena bytes); values (host,
// nplans) receive each plan's final entry (255 = INF).  blocks: 0 = one per SM.  window: plans in
// progress at once (0: all); waiting plans are admitted widest first as running ones finish, which
// keeps the tables of the plans in progress within L2 when the window is small.  Returns
// TG_ERR_TIMEOUT if a block waited longer than its bound for work (the launch still returns).
int tg_batch_run(void *p, void *arena, int blocks, int window, uint32_t *values, void *stream) {
    if (!p || !arena || !values) return set_error(TG_ERR_ARG, "null argument");
    BatchPlan &B = *static_cast<BatchPlan *>(p);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint8_t *d = static_cast<uint8_t *>(B.dev);
    const size_t nj = std::max<size_t>(1, B.jobs.size());
    // counters: taken[nj], done[nj], queue[nj], ready[nj], ctl[8], admission list[nplans]
    std::vector<unsigned> cnt(B.ncnt, 0);
    unsigned *queue = cnt.data() + 2 * nj, *ready = cnt.data() + 3 * nj, *ctl = cnt.data() + 4 * nj;
    unsigned *admit = ctl + 8;
    std::vector<int> order;
    unsigned finished = 0;
    for (int i = 0; i < B.nplans; i++) {
        if (B.first[i] == BJ_NONE) finished++;
        else order.push_back(i);
    }
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return B.width[x] > B.width[y]; });
    const unsigned w = window > 0 ? std::min<unsigned>((unsigned)window, (unsigned)order.size()) : (unsigned)order.size();
    unsigned tail = 0;
    for (unsigned k = 0; k < w; k++) {
        queue[tail] = B.first[order[k]];
        ready[tail] = 1;
        tail++;
    }
    unsigned nadmit = 0;
    for (unsigned k = w; k < order.size(); k++) admit[nadmit++] = B.first[order[k]];
    ctl[0] = 0;
    ctl[1] = tail;
    ctl[2] = finished;
    ctl[3] = 0;
    ctl[4] = 0;
    int e = cuda_check(cudaMemcpyAsync(d + B.off_cnt, cnt.data(), cnt.size() * 4, cudaMemcpyHostToDevice, st), "counters");
    if (e) return e;
    // every plan's start table {0: 0}: the first entry of its first buffer
    for (int i = 0; i < B.nplans; i++) {
        uint64_t a = 0;
        if (B.first[i] != BJ_NONE) a = B.jobs[B.first[i]].src_off;
        else a = B.final_off[i];
        e = cuda_check(cudaMemsetAsync(static_cast<uint8_t *>(arena) + a, 0, 1, st), "start table");
        if (e) return e;
    }
    if (!g_batch_attr) {
        e = cuda_check(cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, BT_TILE_SMEM + 4096), "attr");
        if (e) return e;
        g_batch_attr = true;
    }
    BatchArgs A;
    A.jobs = reinterpret_cast<const BJob *>(d + B.off_jobs);
    A.params = d + B.off_params;
    A.arena = static_cast<uint8_t *>(arena);
    unsigned *dc = reinterpret_cast<unsigned *>(d + B.off_cnt);
    A.taken = dc;
    A.done = dc + nj;
    A.queue = dc + 2 * nj;
    A.ready = dc + 3 * nj;
    A.ctl = dc + 4 * nj;
    A.admit = dc + 4 * nj + 8;
    A.nadmit = nadmit;
    A.nplans = (unsigned)B.nplans;
    A.spin_limit = 20000000ull;          // about 2.5 s of polling at the sleep lengths used
    int grid = blocks > 0 ? blocks : sm_count();
    if (finished < (unsigned)B.nplans) {
        k_batch<<<grid, BT_THREADS, BT_TILE_SMEM + 4096, st>>>(A);
        e = cuda_check(cudaGetLastError(), "batch launch");
        if (e) return e;
    }
    // final entries
    k_batch_values<<<(B.nplans + 255) / 256, 256, 0, st>>>(static_cast<uint8_t *>(arena),
                                                           reinterpret_cast<const uint64_t *>(d + B.off_offs),
                                                           B.nplans, d + B.off_vals);
    e = cuda_check(cudaGetLastError(), "values");
    std::vector<uint8_t> vals(B.nplans);
    unsigned flags = 0;
    if (!e) e = cuda_check(cudaMemcpyAsync(vals.data(), d + B.off_vals, B.nplans, cudaMemcpyDeviceToHost, st), "values");
    if (!e) e = cuda_check(cudaMemcpyAsync(&flags, A.ctl + 3, 4, cudaMemcpyDeviceToHost, st), "flags");
    if (!e) e = cuda_check(cudaStreamSynchronize(st), "batch sync");
    if (e) return e;
    if (flags) return set_error(TG_ERR_TIMEOUT, "a block waited beyond its bound for batch work");
    for (int i = 0; i < B.nplans; i++) values[i] = vals[i];
    return TG_OK;
}

void tg_batch_free(void *p) {
    BatchPlan *B = static_cast<BatchPlan *>(p);
    if (!B) return;
    if (B->dev) cudaFree(B->dev);
    delete B;
}

}  // extern "C"
