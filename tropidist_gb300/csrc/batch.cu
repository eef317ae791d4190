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
#include <functional>
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

// one unit of a job by the whole block: TC = three 64 KB tile buffers, PRM = parameter copy
__device__ void run_unit(const BJob &J, unsigned unit, uint8_t *arena, const uint8_t *params, uint4 *TC, uint4 *PRM) {
    const uint8_t *src = arena + J.src_off;
    uint8_t *dst = arena + J.dst_off;
    if (J.kind == 0 || J.kind == 1) {
        const size_t psize = J.kind == 0 ? sizeof(SweepParams) : sizeof(PassParams);
        const uint4 *g = reinterpret_cast<const uint4 *>(params + J.params_off);
        for (uint32_t i = threadIdx.x; i < (psize + 15) / 16; i += blockDim.x) PRM[i] = __ldcg(g + i);
        __syncthreads();
        if (J.kind == 0) {
            sweep_body<uint8_t>(*reinterpret_cast<const SweepParams *>(PRM), src, dst, TC);
        } else {
            const PassParams &P = *reinterpret_cast<const PassParams *>(PRM);
            const uint64_t t0 = (uint64_t)unit * J.grain;
            const uint64_t nt = P.stream ? (P.ntiles + (1ull << (9 - P.nkt)) - 1) >> (9 - P.nkt) : P.ntiles;
            const uint64_t t1 = t0 + J.grain < nt ? t0 + J.grain : nt;
            if (P.stream) u8_stream_range(P, t0, t1, src, dst, TC);     // a unit: a range of steps
            else if (P.use_groups) u8_pass_range(P, t0, t1, src, dst, TC);
            else
                for (uint64_t t = t0; t < t1; t++) {
                    u8_tile<BT_THREADS>(P, t, src, dst, TC);
                    __syncthreads();
                }
        }
    } else {
        batch_single_op(J, unit, src, dst);
    }
}

// a job descriptor read through L2 (the host may have rewritten the slot since an earlier read)
__device__ __forceinline__ BJob load_job(const BJob *p) {
    BJob J;
    const uint4 *s = reinterpret_cast<const uint4 *>(p);
    uint4 *d = reinterpret_cast<uint4 *>(&J);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(BJob) / 16); i++) d[i] = __ldcg(s + i);
    return J;
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
        run_unit(J, s_unit, A.arena, A.params, TC, PRM);
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

// work items of a fused pass: tiles, or steps of 512 >> nk tiles in the streaming form
static uint64_t pass_units(const PassParams &pp) {
    return pp.stream ? (pp.ntiles + (1ull << (9 - pp.nkt)) - 1) >> (9 - pp.nkt) : pp.ntiles;
}
// items per unit: at least 16, about one unit per SM for a lone plan
static uint32_t pass_grain(uint64_t nt) {
    return (uint32_t)std::min<uint64_t>(nt, std::max<uint64_t>(16, (nt + sm_count() - 1) / sm_count()));
}

static_assert(sizeof(SweepParams) <= 4096 && sizeof(PassParams) <= 4096, "job parameters exceed their 4 KB copy");
static_assert(sizeof(BJob) % 16 == 0, "job descriptors are read as 16-byte words");

static bool g_batch_attr = false;


// ------------------------------------------------------------------ continuous serving
// The same units in a long-lived launch whose work arrives while it runs.  Device memory holds a
// pool of job descriptors, parameters and counters (slots reused by the host), the job queue
// (circular over the job pool), and a mailbox of admitted plans' first jobs that the host fills by
// DMA on a copy stream (entry first, then the mailbox tail).  A block that looks for work first
// moves mailbox entries into the queue, then takes a unit; a plan's last unit sets its done flag.
// A block that finds nothing for `idle_limit` polls leaves; the host relaunches the kernel when
// new work arrives, and all state persists across launches.
struct ServerArgs {
    const BJob *jobs;
    const uint8_t *params;
    uint8_t *arena;
    unsigned *taken, *done, *queue, *ready;
    unsigned *ctl;           // 0 queue head, 1 queue tail, 3 error, 4 mailbox head, 5 stop, 6 mailbox tail
    const unsigned *mbox;
    unsigned *plan_done;     // per plan slot: 0 running, 0x100 | final entry when done
    unsigned jcap, mcap;
    unsigned long long idle_limit;
};

__device__ void server_push(const ServerArgs &A, unsigned j) {
    const unsigned slot = atomicAdd(A.ctl + 1, 1u);
    A.queue[slot % A.jcap] = j;
    __threadfence();
    atomicExch(A.ready + slot % A.jcap, slot + 1u);    // the position, so a slot needs no clearing
}

// thread 0: state 0 job, 1 leave (stop flag or idle)
__device__ void server_grab(const ServerArgs &A, int &state, unsigned &job, unsigned &unit, BJob &J) {
    unsigned long long idle = 0;
    while (idle < A.idle_limit) {
        if (ld_volatile(A.ctl + 5)) break;
        const unsigned mt = ld_volatile(A.ctl + 6), mh = ld_volatile(A.ctl + 4);
        if (mh < mt) {
            if (atomicCAS(A.ctl + 4, mh, mh + 1) == mh) {
                __threadfence();
                server_push(A, ld_volatile(A.mbox + mh % A.mcap));
            }
            continue;
        }
        const unsigned h = ld_volatile(A.ctl + 0), t = ld_volatile(A.ctl + 1);
        if (h < t) {
            if (ld_volatile(A.ready + h % A.jcap) != h + 1u) { __nanosleep(64); idle++; continue; }
            __threadfence();
            const unsigned j = ld_volatile(A.queue + h % A.jcap);
            J = load_job(A.jobs + j);
            const unsigned u = atomicAdd(A.taken + j, 1u);
            if (u < J.nunits) { state = 0; job = j; unit = u; __threadfence(); return; }
            atomicCAS(A.ctl + 0, h, h + 1);
            continue;
        }
        __nanosleep(256);
        idle++;
    }
    state = 1;
}

__global__ void __launch_bounds__(BT_THREADS, 1) k_server(const __grid_constant__ ServerArgs A) {
    extern __shared__ uint4 smem_raw[];
    uint4 *TC = smem_raw;
    uint4 *PRM = smem_raw + (BT_TILE_SMEM / 16);
    __shared__ int s_state;
    __shared__ unsigned s_job, s_unit;
    __shared__ BJob s_J;
    for (;;) {
        if (threadIdx.x == 0) {
            int st = 1;
            unsigned j = 0, u = 0;
            BJob J;
            server_grab(A, st, j, u, J);
            s_state = st;
            s_job = j;
            s_unit = u;
            if (st == 0) s_J = J;
        }
        __syncthreads();
        if (s_state != 0) break;
        const BJob J = s_J;
        run_unit(J, s_unit, A.arena, A.params, TC, PRM);
        __threadfence();
        __syncthreads();
        if (threadIdx.x == 0) {
            const unsigned prev = atomicAdd(A.done + s_job, 1u);
            if (prev + 1 == J.nunits) {
                if (J.next != BJ_NONE) {
                    server_push(A, J.next);
                } else {
                    // the plan's result: entry 0 of the last job's output, written (and fenced) by
                    // the block that ran unit 0 before its completion count
                    __threadfence();
                    const unsigned v = *reinterpret_cast<volatile const uint8_t *>(A.arena + J.dst_off);
                    atomicExch(A.plan_done + J.plan, 0x100u | v);
                }
            }
        }
        __syncthreads();
    }
}

// first-fit allocator over [0, cap) in units of `align`
struct RangeAlloc {
    uint64_t cap = 0, align = 1;
    std::vector<std::pair<uint64_t, uint64_t>> free;   // (offset, size), sorted by offset
    void init(uint64_t c, uint64_t a) { cap = c; align = a; free.assign(1, {0, c}); }
    bool take(uint64_t n, uint64_t &off) {
        n = (n + align - 1) / align * align;
        for (size_t i = 0; i < free.size(); i++) {
            if (free[i].second >= n) {
                off = free[i].first;
                free[i].first += n;
                free[i].second -= n;
                if (!free[i].second) free.erase(free.begin() + i);
                return true;
            }
        }
        return false;
    }
    void give(uint64_t off, uint64_t n) {
        n = (n + align - 1) / align * align;
        auto it = std::lower_bound(free.begin(), free.end(), std::make_pair(off, (uint64_t)0));
        it = free.insert(it, {off, n});
        size_t i = it - free.begin();
        if (i + 1 < free.size() && free[i].first + free[i].second == free[i + 1].first) {
            free[i].second += free[i + 1].second;
            free.erase(free.begin() + i + 1);
        }
        if (i > 0 && free[i - 1].first + free[i - 1].second == free[i].first) {
            free[i - 1].second += free[i].second;
            free.erase(free.begin() + i);
        }
    }
};

struct ServedPlan {
    bool live = false, done = false, reported = false, tail_seen = false;
    uint64_t arena_off = 0, arena_bytes = 0, job0 = 0, njobs = 0, prm_off = 0, prm_bytes = 0;
    unsigned value = 0;
    unsigned tail_at_done = 0;     // queue tail read after the plan finished
};

struct Server {
    uint8_t *arena = nullptr;
    void *dev = nullptr;
    unsigned jcap = 0, mcap = 0, pcap = 0;
    uint64_t prm_cap = 0;
    BJob *d_jobs = nullptr;
    uint8_t *d_params = nullptr;
    unsigned *d_taken = nullptr, *d_done = nullptr, *d_queue = nullptr, *d_ready = nullptr, *d_ctl = nullptr;
    unsigned *d_mbox = nullptr, *d_plan_done = nullptr;
    cudaStream_t ks = nullptr, cs = nullptr;
    RangeAlloc arena_a, job_a, prm_a;
    std::vector<ServedPlan> plans;
    std::vector<unsigned> free_slots;    // kept sorted, highest first: low slots are reused first
    unsigned mbox_tail = 0;
    int blocks = 0;
    bool launched = false;
    unsigned *h_buf = nullptr;           // pinned: plan_done flags, then the control words
};

static int server_launch(Server &S) {
    if (S.launched && cudaStreamQuery(S.ks) == cudaErrorNotReady) return TG_OK;
    cudaGetLastError();
    ServerArgs A;
    A.jobs = S.d_jobs;
    A.params = S.d_params;
    A.arena = S.arena;
    A.taken = S.d_taken;
    A.done = S.d_done;
    A.queue = S.d_queue;
    A.ready = S.d_ready;
    A.ctl = S.d_ctl;
    A.mbox = S.d_mbox;
    A.plan_done = S.d_plan_done;
    A.jcap = S.jcap;
    A.mcap = S.mcap;
    A.idle_limit = 20000ull;        // about 5-10 ms of polling without work, then the blocks leave
    static bool attr = false;
    if (!attr) {
        const int e = cuda_check(cudaFuncSetAttribute(k_server, cudaFuncAttributeMaxDynamicSharedMemorySize, BT_TILE_SMEM + 4096), "attr");
        if (e) return e;
        attr = true;
    }
    k_server<<<S.blocks, BT_THREADS, BT_TILE_SMEM + 4096, S.ks>>>(A);
    S.launched = true;
    return cuda_check(cudaGetLastError(), "server launch");
}


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
                    // large units amortise the per-unit overhead; concurrency comes from the other plans
                    const uint64_t nt = pass_units(S.pp);
                    J.grain = pass_grain(nt);
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
// polls of one wait for work before a block gives up (0: the default, about 2.5 s)
static unsigned long long g_batch_spin = 0;

int tg_batch_set_spin_limit(uint64_t polls) {
    g_batch_spin = polls;
    return TG_OK;
}

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
    A.spin_limit = g_batch_spin ? g_batch_spin : 20000000ull;   // about 2.5 s of polling by default
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

// ---------------------------------------------------------------- continuous serving
// Pools: jobs (jcap descriptors), parameters (prm_bytes), plan slots (plan_cap).  arena: device
// tables of the plans in progress (caller-owned, arena_bytes).
void *tg_server_create(void *arena, uint64_t arena_bytes, int jcap, int64_t prm_bytes, int plan_cap, int blocks,
                       int *status) {
    int st = TG_OK;
    Server *S = nullptr;
    if (!arena || !arena_bytes || jcap <= 0 || prm_bytes <= 0 || plan_cap <= 0)
        st = set_error(TG_ERR_ARG, "bad server arguments");
    if (!st) {
        S = new Server();
        S->arena = static_cast<uint8_t *>(arena);
        S->jcap = (unsigned)jcap;
        S->mcap = S->pcap = (unsigned)plan_cap;
        S->prm_cap = (uint64_t)prm_bytes;
        S->blocks = blocks > 0 ? blocks : sm_count();
        const size_t o_prm = align_up((size_t)jcap * sizeof(BJob), 256);
        const size_t o_cnt = align_up(o_prm + (size_t)prm_bytes, 256);
        const size_t ncnt = 4 * (size_t)jcap + 8 + 2 * (size_t)plan_cap;
        if (cudaMalloc(&S->dev, o_cnt + ncnt * 4) != cudaSuccess) {
            cudaGetLastError();
            S->dev = nullptr;
            st = set_error(TG_ERR_NOMEM, "server pools");
        }
        if (!st) {
            uint8_t *d = static_cast<uint8_t *>(S->dev);
            S->d_jobs = reinterpret_cast<BJob *>(d);
            S->d_params = d + o_prm;
            unsigned *c = reinterpret_cast<unsigned *>(d + o_cnt);
            S->d_taken = c;
            S->d_done = c + jcap;
            S->d_queue = c + 2 * (size_t)jcap;
            S->d_ready = c + 3 * (size_t)jcap;
            S->d_ctl = c + 4 * (size_t)jcap;
            S->d_mbox = S->d_ctl + 8;
            S->d_plan_done = S->d_mbox + plan_cap;
            st = cuda_check(cudaMemset(c, 0, ncnt * 4), "server counters");
        }
        if (!st) st = cuda_check(cudaStreamCreateWithFlags(&S->ks, cudaStreamNonBlocking), "server stream");
        if (!st) st = cuda_check(cudaStreamCreateWithFlags(&S->cs, cudaStreamNonBlocking), "copy stream");
        if (!st) st = cuda_check(cudaMallocHost(&S->h_buf, ((size_t)plan_cap + 8) * 4), "server host buffer");
        if (!st) {
            S->arena_a.init(arena_bytes, 256);
            S->job_a.init((uint64_t)jcap, 1);
            S->prm_a.init((uint64_t)prm_bytes, 16);
            S->plans.assign(plan_cap, ServedPlan());
            for (int k = plan_cap - 1; k >= 0; k--) S->free_slots.push_back((unsigned)k);
        }
        if (st) {
            if (S->ks) cudaStreamDestroy(S->ks);
            if (S->cs) cudaStreamDestroy(S->cs);
            if (S->h_buf) cudaFreeHost(S->h_buf);
            if (S->dev) cudaFree(S->dev);
            delete S;
            S = nullptr;
        }
    }
    if (status) *status = st;
    return S;
}

// Admits one plan (op stream of nops rows (code, a, b), uint8 tables).  Returns its slot, or
// TG_ERR_NOMEM when the arena, the pools or the plan slots have no room now (collect finished
// plans with tg_server_poll and retry), or another negative status.
static int server_submit(Server &S, const DensePlan &P);

int tg_server_submit(void *p, const int64_t *ops, int64_t nops) {
    if (!p || (!ops && nops)) return set_error(TG_ERR_ARG, "null argument");
    Server &S = *static_cast<Server *>(p);
    if (S.free_slots.empty()) return TG_ERR_NOMEM;
    DensePlan P;
    const int st = build_dense_plan(ops, nops, 1, nullptr, 0, P);
    if (st) return st;
    return server_submit(S, P);
}

// Admits a plan scheduled ahead of time by tg_dense_plan (uint8 entries); same returns as
// tg_server_submit.  The plan handle stays the caller's.
int tg_server_submit_plan(void *p, void *plan) {
    if (!p || !plan) return set_error(TG_ERR_ARG, "null argument");
    Server &S = *static_cast<Server *>(p);
    const DensePlan &P = *static_cast<const DensePlan *>(plan);
    if (P.eb != 1) return set_error(TG_ERR_ARG, "served plans have uint8 entries");
    if (S.free_slots.empty()) return TG_ERR_NOMEM;
    return server_submit(S, P);
}

static int server_submit(Server &S, const DensePlan &P) {
    int st = TG_OK;
    for (const Seg &G : P.segs)
        if ((G.kind == 0 && G.sp.max_bits > 15) || (G.kind == 1 && G.pp.d > 16))
            return set_error(TG_ERR_TOO_BIG, "served plans need sweeps of <= 15 bits and tiles of <= 16 bits");
    const unsigned slot = S.free_slots.back();
    ServedPlan &R = S.plans[slot];
    R = ServedPlan();
    if (P.segs.empty()) {              // nothing to run: the start table {0: 0} is the result
        S.free_slots.pop_back();
        R.live = R.done = true;
        R.tail_seen = true;
        R.value = 0;
        return (int)slot;
    }
    // parameter blob and jobs
    std::vector<uint8_t> prm;
    std::vector<BJob> jobs(P.segs.size());
    const uint64_t tb = align_up((size_t)1 << P.peak_bits, 256);
    R.arena_bytes = 2 * tb;
    if (!S.arena_a.take(R.arena_bytes, R.arena_off)) return TG_ERR_NOMEM;
    for (const Seg &G : P.segs) {
        const size_t n = G.kind == 0 ? sizeof(SweepParams) : G.kind == 1 ? sizeof(PassParams) : 0;
        if (n) prm.resize(align_up(prm.size(), 16) + n);
    }
    R.prm_bytes = std::max<size_t>(16, prm.size());
    R.njobs = jobs.size();
    if (!S.job_a.take(R.njobs, R.job0)) {
        S.arena_a.give(R.arena_off, R.arena_bytes);
        return TG_ERR_NOMEM;
    }
    if (!S.prm_a.take(R.prm_bytes, R.prm_off)) {
        S.arena_a.give(R.arena_off, R.arena_bytes);
        S.job_a.give(R.job0, R.njobs);
        return TG_ERR_NOMEM;
    }
    S.free_slots.pop_back();
    R.live = true;
    const uint64_t a = R.arena_off, b = a + tb;
    size_t poff = 0;
    int cur = 0;
    for (size_t k = 0; k < P.segs.size(); k++) {
        const Seg &G = P.segs[k];
        BJob &J = jobs[k];
        memset(&J, 0, sizeof(J));
        J.plan = (int)slot;
        J.next = k + 1 < P.segs.size() ? (unsigned)(R.job0 + k + 1) : BJ_NONE;
        J.src_off = cur ? b : a;
        J.dst_off = cur ? a : b;
        if (G.kind == 0) {
            J.kind = 0;
            J.nunits = 1;
            poff = align_up(poff, 16);
            memcpy(prm.data() + poff, &G.sp, sizeof(SweepParams));
            J.params_off = R.prm_off + poff;
            poff += sizeof(SweepParams);
        } else if (G.kind == 1) {
            J.kind = 1;
            const uint64_t nt = pass_units(G.pp);
            J.grain = pass_grain(nt);
            J.nunits = (uint32_t)((nt + J.grain - 1) / J.grain);
            poff = align_up(poff, 16);
            memcpy(prm.data() + poff, &G.pp, sizeof(PassParams));
            J.params_off = R.prm_off + poff;
            poff += sizeof(PassParams);
        } else {
            J.kind = 2;
            J.bits = G.w_in;
            J.op_code = G.op_code;
            J.op_a = G.op_a;
            J.op_b = G.op_b;
            const uint64_t chunks = std::max<uint64_t>(1, ((uint64_t)1 << G.w_in) >> 4);
            J.nunits = (uint32_t)((chunks + BJ_UNIT_CHUNKS - 1) / BJ_UNIT_CHUNKS);
        }
        cur ^= 1;
    }
    if ((P.final_buf ? b : a) != jobs.back().dst_off) return set_error(TG_ERR_STATE, "plan result buffer mismatch");
    // descriptors, counters, start table, then the mailbox entry and tail (stream order on the copy
    // stream makes everything before the tail visible before the kernel can see the entry)
    unsigned *hb = S.h_buf;
    const unsigned first = (unsigned)R.job0;
    cudaStream_t cs = S.cs;
    st = cuda_check(cudaMemcpyAsync(S.d_jobs + R.job0, jobs.data(), jobs.size() * sizeof(BJob), cudaMemcpyHostToDevice, cs), "server jobs");
    if (!st && !prm.empty())
        st = cuda_check(cudaMemcpyAsync(S.d_params + R.prm_off, prm.data(), prm.size(), cudaMemcpyHostToDevice, cs), "server params");
    if (!st) st = cuda_check(cudaMemsetAsync(S.d_taken + R.job0, 0, R.njobs * 4, cs), "taken");
    if (!st) st = cuda_check(cudaMemsetAsync(S.d_done + R.job0, 0, R.njobs * 4, cs), "done");
    if (!st) st = cuda_check(cudaMemsetAsync(S.d_plan_done + slot, 0, 4, cs), "plan flag");
    if (!st) st = cuda_check(cudaMemsetAsync(S.arena + a, 0, 1, cs), "start table");
    if (!st) {
        hb[0] = first;
        hb[1] = S.mbox_tail + 1;
        st = cuda_check(cudaMemcpyAsync(S.d_mbox + S.mbox_tail % S.mcap, hb, 4, cudaMemcpyHostToDevice, cs), "mailbox");
    }
    if (!st) st = cuda_check(cudaMemcpyAsync(S.d_ctl + 6, hb + 1, 4, cudaMemcpyHostToDevice, cs), "mailbox tail");
    if (!st) st = cuda_check(cudaStreamSynchronize(cs), "submit sync");
    if (st) return st;
    S.mbox_tail++;
    st = server_launch(S);
    return st ? st : (int)slot;
}

// Finished plans since the last call: up to `max` (slot, final entry) pairs into slots/values
// (host arrays).  Returns how many, or a negative status.  Frees a finished plan's tables at once
// and its descriptors once the queue head has passed every position the plan used.
int tg_server_poll(void *p, int *slots, uint32_t *values, int max) {
    if (!p || (max > 0 && (!slots || !values))) return set_error(TG_ERR_ARG, "null argument");
    Server &S = *static_cast<Server *>(p);
    unsigned hi = 0;
    bool running = false;
    for (unsigned k = 0; k < S.pcap; k++)
        if (S.plans[k].live) {
            hi = k + 1;
            running |= !S.plans[k].done;
        }
    unsigned *flags = S.h_buf, *ctl = S.h_buf + S.pcap;
    int st = TG_OK;
    if (hi) st = cuda_check(cudaMemcpyAsync(flags, S.d_plan_done, (size_t)hi * 4, cudaMemcpyDeviceToHost, S.cs), "plan flags");
    // after the flags: a tail read here is at or past the last push of every plan seen finished
    if (!st) st = cuda_check(cudaMemcpyAsync(ctl, S.d_ctl, 8 * 4, cudaMemcpyDeviceToHost, S.cs), "control words");
    if (!st) st = cuda_check(cudaStreamSynchronize(S.cs), "poll sync");
    if (st) return st;
    if (ctl[3]) return set_error(TG_ERR_TIMEOUT, "a server block waited beyond its bound");
    const cudaError_t q = cudaStreamQuery(S.ks);
    if (q != cudaSuccess && q != cudaErrorNotReady) return cuda_check(q, "server kernel");
    int n = 0;
    for (unsigned k = 0; k < hi; k++) {
        ServedPlan &R = S.plans[k];
        if (!R.live) continue;
        if (!R.done && (flags[k] & 0x100u)) {
            R.done = true;
            R.value = flags[k] & 0xFFu;
            R.tail_at_done = ctl[1];
            S.arena_a.give(R.arena_off, R.arena_bytes);
        } else if (R.done && !R.tail_seen && R.njobs && (int)(ctl[0] - R.tail_at_done) >= 0) {
            // a later poll: no block can still be reading these descriptors
            R.tail_seen = true;
            S.job_a.give(R.job0, R.njobs);
            S.prm_a.give(R.prm_off, R.prm_bytes);
        }
        if (R.done && !R.reported && n < max) {
            slots[n] = (int)k;
            values[n] = R.value;
            n++;
            R.reported = true;
        }
        if (R.done && R.reported && R.tail_seen) {
            R.live = false;
            S.free_slots.insert(std::upper_bound(S.free_slots.begin(), S.free_slots.end(), k, std::greater<unsigned>()), k);
        }
    }
    if (running) {
        bool undone = false;
        for (unsigned k = 0; k < hi; k++) undone |= S.plans[k].live && !S.plans[k].done;
        if (undone) {
            st = server_launch(S);      // blocks that idled out leave; new work brings them back
            if (st) return st;
        }
    }
    return n;
}

// Makes the kernel's blocks leave and waits for them.
int tg_server_stop(void *p) {
    if (!p) return set_error(TG_ERR_ARG, "null server");
    Server &S = *static_cast<Server *>(p);
    S.h_buf[S.pcap] = 1;
    int st = cuda_check(cudaMemcpyAsync(S.d_ctl + 5, S.h_buf + S.pcap, 4, cudaMemcpyHostToDevice, S.cs), "stop flag");
    if (!st) st = cuda_check(cudaStreamSynchronize(S.cs), "stop sync");
    if (!st) st = cuda_check(cudaStreamSynchronize(S.ks), "server drain");
    if (!st) {
        S.h_buf[S.pcap] = 0;
        st = cuda_check(cudaMemcpyAsync(S.d_ctl + 5, S.h_buf + S.pcap, 4, cudaMemcpyHostToDevice, S.cs), "stop flag");
        if (!st) st = cuda_check(cudaStreamSynchronize(S.cs), "stop sync");
    }
    return st;
}

void tg_server_free(void *p) {
    Server *S = static_cast<Server *>(p);
    if (!S) return;
    tg_server_stop(S);
    cudaStreamDestroy(S->ks);
    cudaStreamDestroy(S->cs);
    cudaFreeHost(S->h_buf);
    cudaFree(S->dev);
    delete S;
}

}  // extern "C"
