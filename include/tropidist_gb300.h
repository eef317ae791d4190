/* libtropigpu: GB300 (sm_103a) Rank DP evaluators behind a C ABI.
 *
 * Every pointer named T, buf_* or *_dev is a DEVICE pointer (cudaMalloc / torch CUDA memory);
 * hist, value, ops and info are HOST pointers.  Calls are stream-ordered: the reference-style
 * per-op functions (dp_*) run on the stream set by tg_set_stream (default: the legacy default
 * stream) and return before the GPU finishes, except dp_hist, which waits for its result.
 * Status codes: 0 ok, -1 bad argument, -2 CUDA error, -3 out of device memory, -4 beyond a
 * documented maximum, -5 a bounded device wait ran out, -6 wrong state; tg_last_error() has the
 * text of the last failure of the calling thread.  No entry point exits the process or traps
 * the device.
 */
#ifndef TROPIDIST_GB300_H
#define TROPIDIST_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- library */
int tg_version(void);
const char *tg_last_error(void);
int tg_sm_count(void);
void tg_set_stream(void *stream);   /* cudaStream_t used by the dp_* per-op functions */

/* ---------------------------------------------------------------- dense Rank DP, per op
 * Drop-in for the ctypes binding of cdist/viterbi.c (cdist/kernel.py:52-69), on device tables
 * of n = 2^bits uint8 entries, INF = 255, saturating additions. */
void dp_update(uint8_t *T, uint64_t n, uint64_t h);                 /* cdist/viterbi.c:73  */
void dp_expand_update(uint8_t *T, uint64_t n, uint64_t hl);         /* cdist/viterbi.c:122 (T holds 2n) */
uint64_t dp_select(uint8_t *T, uint64_t n, int pos, int target);    /* cdist/viterbi.c:155 (in place) */
void dp_fill(uint8_t *T, uint64_t n, uint8_t v);                    /* cdist/viterbi.c:174 */
void dp_hist(const uint8_t *T, uint64_t n, uint64_t *hist);         /* cdist/viterbi.c:182 (hist: host[256]) */
int dp_num_threads(void);                                           /* cdist/viterbi.c:195 (SM count) */
void dp_update_w(uint8_t *T, uint64_t n, uint64_t h, int w);        /* cdist/viterbi.c:204 */

/* uint16 tables (INF = 65535), the same rules; no counterpart in the reference, which has
 * 8-bit dense tables only (cdist/kernel.py:13) */
int dp16_update(uint16_t *T, uint64_t n, uint64_t h, int w);
int dp16_expand_update(uint16_t *T, uint64_t n, uint64_t hl, int w);
uint64_t dp16_select(uint16_t *T, uint64_t n, int pos, int target);

/* ---------------------------------------------------------------- dense Rank DP, whole plan
 * Replaces the executor loop of cdist/kernel.py:94-138 (run_plan).  ops: nops rows of int64
 * (code, a, b): (0, 0, 0) expand, (1, mask, w) update, (2, pos, target) select, i.e. the
 * trellis Plan.ops of cdist/trellis.py:125-182 encoded row by row.  entry_bytes: 1 (uint8) or
 * 2 (uint16).  buf_a and buf_b each hold 2^peak_bits entries; the tables ping-pong between them.
 * ckpt_ops: op counts k after which the table (2^width(k) entries) is copied to ckpt_bufs[i]. */
void *tg_dense_plan(const int64_t *ops, int64_t nops, int entry_bytes, const int64_t *ckpt_ops,
                    int64_t nckpt, int *status);
/* a plan of ops that follow a table of width w_start (canonical order, put in buffer a by the
 * caller before tg_dense_execute; no counterpart in the reference, which never restarts a sweep); it
 * may end at any width, with its final table (canonical order) in the final buffer.  Used to
 * recompute segments between checkpoints for the witness traceback. */
void *tg_dense_plan_from(const int64_t *ops, int64_t nops, int entry_bytes, int w_start, const int64_t *ckpt_ops,
                         int64_t nckpt, int *status);
int tg_dense_plan_info(void *plan, int64_t *info, int ninfo);
/* info: peak_bits, segments, fused passes, shared-memory sweeps, final buffer (0 a / 1 b),
 *       update ops, pass bytes, sweep bytes */
/* per segment 8 int64: kind (0 sweep, 1 fused tile pass, 2 one-op pass, 3 coset-streaming pass),
 * width in, width out, ops done, tile bits, updates, register groups (kind 3: residual updates,
 * + 16 when coset members are word-permuted, + 32 with a lane dimension, + 64 when its update has
 * an in-chunk part), store mode */
int tg_dense_plan_segments(void *plan, int64_t *out, int64_t maxseg);
void tg_dense_plan_free(void *plan);
int tg_dense_execute(void *plan, void *buf_a, void *buf_b, void **ckpt_bufs, void *stream);
int tg_dense_result(void *plan, void *buf_a, void *buf_b, uint32_t *value, void *stream);
/* execute with a CUDA event pair around every launch (on `stream`), waits for the end; out[12]:
 * for shared-memory sweeps, fused tile passes, one-op passes and coset-streaming passes:
 * launches, total ms, table bytes (nout < 12 truncates) */
int tg_dense_execute_timed(void *plan, void *buf_a, void *buf_b, void *stream, double *out, int nout);
/* per-segment launch times (ms) of the plan's last timed execution; returns the count */
int tg_dense_segment_ms(void *plan, float *out, int64_t maxseg);
int tg_dense_run(const int64_t *ops, int64_t nops, int entry_bytes, void *buf_a, void *buf_b,
                 uint32_t *value, void *stream);
int tg_dense_set_tuning(int dmax8, int dmax16, int sweep_bits8, int sweep_bits16);
/* coset-streaming passes: update span (3, or 4 with a lane-pair dimension) and the span of passes
 * in which an in-chunk row closes (<= span, 2 or 3); default 3, 2 */
int tg_dense_set_stream_span(int span, int span_sel);

/* Allocation-free whole-plan run (uint8 tables).  No counterpart in the reference: its C kernels
 * never allocate, because numpy owns the one table buffer (cdist/kernel.py:101-103), whereas the
 * GPU executor needs a second, ping-pong table.  This variant is for callers that cannot allocate
 * device memory, such as a runtime that owns the whole device-memory budget, or a caller on a stream
 * where a synchronizing cudaMalloc would stall concurrent work.  It takes the second table from a
 * 4 MiB array held in device memory by the library itself.  Limits and rules:
 *   - plans up to peak_bits = 22; wider plans return -4 (TG_ERR_TOO_BIG) and launch nothing;
 *   - table_dev (device, >= 2^peak_bits bytes) is the caller's first table and is overwritten;
 *   - value (host) receives the final entry (255 = INF), and the call waits for it;
 *   - no device memory is allocated or freed;
 *   - the first call on each device looks up the array's device address
 *     (cudaGetSymbolAddress); make that first call before any stream capture;
 *   - every call shares the one array, so calls that overlap on the GPU (other streams, other
 *     host threads) race: run them one after another. */
int tg_dense_run_noalloc(const int64_t *ops, int64_t nops, uint8_t *table_dev, uint64_t table_entries,
                         uint32_t *value, void *stream);
/* tg_dense_plan + tg_dense_execute in one call: each segment is launched on `stream` as soon as the
 * scheduler emits it, so the first passes run while the rest of the plan is scheduled.  Returns
 * the plan (for tg_dense_result, tg_dense_plan_info and tg_dense_plan_free; no checkpoints, not to be
 * executed again); NULL and *status on an error (the launches made so far stay queued).  Both
 * buffers hold buf_entries entries; an op stream wider than that launches nothing. */
void *tg_dense_plan_execute(const int64_t *ops, int64_t nops, int entry_bytes, void *buf_a, void *buf_b,
                            uint64_t buf_entries, void *stream, int *status);
/* Witness of a small plan in one launch (the traceback of cdist/auto.py:126-182 on the device): one
 * block applies the ops (HOST int64 [n][3] as tg_dense_plan, entries of eb bytes) keeping every
 * table of the sweep in `tables` (DEVICE, tg_dense_witness_bytes(ops, n, eb) bytes), then one
 * thread walks back from the final entry.  out_dev: DEVICE int32 [3 + out_cap] = final entry,
 * number of used updates, their op indices (last op first), status (0 ok, 1 bad op stream or
 * storage, 2 the walk lost the path).  tg_dense_witness_bytes returns -1 for a bad op stream. */
int64_t tg_dense_witness_bytes(const int64_t *ops, int64_t n, int eb);
int tg_dense_witness_small(const int64_t *ops, int64_t n, int eb, void *tables, uint64_t table_bytes,
                           int32_t *out_dev, int64_t out_cap, void *stream);
/* Runs a scheduled plan on HOST buffers with the launch parameters and index arithmetic of the
 * kernels; for checking the scheduler on a machine without a GPU.  Not an evaluator. */
int tg_debug_emulate_dense(void *plan, void *host_a, void *host_b, void **ckpt_host);

/* ---------------------------------------------------------------- sparse Rank DP (device tables)
 * A table: n packed states key | value << 56 (key = row-slot parities, <= 56 slots; value 0..254),
 * the format of the reference's C tables (cdist/sparse_dp.c:3-4), in a device array, plus a device
 * index of 2^lg slots (open addressing, empty slot = all ones).  counters: device uint64[4] =
 * new keys, changed states, error flags (1 index full, 2 changed list full, 4 array full), states
 * written.  These replace sp_candidates + sp_merge (cdist/sparse_dp.c:118-202, bound by
 * cdist/sparse_dp.py:487-497) with one step on device tables. */
int tg_sp_clear(void *H, uint64_t cap, void *stream);
int tg_sp_step(const void *A, uint64_t n, const void *Hold, int lg_old, void *Hnew, int lg_new, void *Anew,
               uint64_t anew_cap, void *changed, uint64_t changed_cap, uint64_t upd, uint64_t sel_mask,
               uint64_t sel_bits, int cap, int keep_below, int w, int want_changed, int use_h, int K, int ncls,
               const uint64_t *masks, const int64_t *weights, int64_t extra, uint64_t tmask, void *counters,
               void *stream);
int tg_sp_build(const void *A, uint64_t n, void *H, int lg, int below, void *kept, void *counters, void *stream);
/* replaces sp_join (cdist/sparse_dp.c:207-236): result (device uint64) = min (total << 56 | fkey) */
int tg_sp_join(const void *F, uint64_t nf, const void *Hb, int lgb, uint64_t tmask, void *result, void *stream);
int tg_sp_lookup(const void *H, int lg, const void *keys, uint64_t n, void *vals, void *stream);
/* A run of column steps in one call (no counterpart in the reference, whose Python loop calls
 * sp_candidates + sp_merge once per column): steps described by spec rows (host int64[16]), tables
 * in caller-provided scratch, kept tables copied to a caller-provided arena, joins against backward
 * indexes accumulated per step on the device; see csrc/sparse.cu for the fields.  Returns nsteps,
 * or the step where scratch / arena ran out (need[0] states, need[1] bytes; run again). */
int64_t tg_sp_walk_scratch_bytes(uint64_t cap_n);
/* host planning (no GPU): GF(2) rank of the first i columns of an order, i = 0..ncols
 * (cdist/trellis.py:20-36); columns as CSR lists of rows */
int tg_rank_profile(int ncols, int nrows, const int64_t *col_ptr, const int32_t *col_rows, const int32_t *order,
                    int32_t *out);
/* host planning (no GPU): the op stream of one dense query (the loop of cdist/trellis.py:147-182)
 * from nrows bitset rows of `words` uint64 over column positions, the target row last; weights per
 * position or NULL.  ops: int64 [cap][3] (expand 0,0,0 / update 1,mask,w / select 2,pos,target);
 * widths: int32 [ncols]; columns: int32 [cap] (position of each update); out: ops, updates, peak.
 * Returns 0, a negative status (-4: a mask beyond 63 rows), or the op count needed when > cap. */
int tg_make_plan(int nrows, int ncols, int words, const uint64_t *rows, const int64_t *weights, int64_t *ops,
                 int64_t cap, int32_t *widths, int32_t *columns, int64_t *out);
/* host planning (no GPU): the lookahead classes of every cut (the per-cut loop of
 * cdist/sparse_dp.py:148-192), CSR inputs; see csrc/sparse.cu */
int tg_sp_bound_data(int N, int nrows, const int64_t *row_ptr, const int32_t *row_cols, const int64_t *col_ptr,
                     const int32_t *col_rows, const int64_t *act_ptr, const int32_t *act_rows, const int32_t *row_start,
                     const int32_t *row_end, const int32_t *slot, int L, int forward, int maxc, int32_t *ncls,
                     uint64_t *masks, int64_t *weights, int64_t *extra);
/* the same for row slots beyond one word: masks uint64 [N + 1][maxc][words] (slot s in word s / 64) */
int tg_sp_bound_data_wide(int N, int nrows, const int64_t *row_ptr, const int32_t *row_cols, const int64_t *col_ptr,
                          const int32_t *col_rows, const int64_t *act_ptr, const int32_t *act_rows,
                          const int32_t *row_start, const int32_t *row_end, const int32_t *slot, int L, int forward,
                          int maxc, int words, int32_t *ncls, uint64_t *masks, int64_t *weights, int64_t *extra);
int tg_sp_walk(int nsteps, const int64_t *spec, const uint64_t *masks, const int64_t *weights, int stride, int K,
               const void *A0, uint64_t n0, const void *H0, int lg0, void *scratch, uint64_t cap_n, void *arena,
               uint64_t arena_bytes, int64_t *out, void *join_results, int64_t *need, void *counters, void *stream);
/* replaces sp_hist (cdist/sparse_dp.c:239-242): hist is a device uint64[256] */
int tg_sp_hist(const void *A, uint64_t n, void *hist, void *stream);

/* ---------------------------------------------------------------- sparse Rank DP, wide states
 * States of W = 1..8 uint64 words (up to 512 row slots; the reference holds at most 56 in C and 64 in
 * numpy, cdist/sparse_dp.c:3-4, cdist/sparse_dp.py:97-98, and refuses wider trellises).  A table:
 * keys DEVICE uint64 [W][stride] (word w of state i at w * stride + i), vals DEVICE uint8 [stride],
 * index DEVICE uint64 [2^lg] (value << 56 | state, empty = all ones).  Masks and states passed by
 * the host are HOST uint64 [W]; lookahead masks HOST uint64 [ncls][W] (ncls <= 32).  counters:
 * DEVICE uint64 [4] = states written, changed states, error flags (1 index full, 2 changed list
 * full, 4 table full), unused.
 * One column step, the rule of sp_candidates + sp_merge (cdist/sparse_dp.c:118-202) with a column
 * weight w: staging keys/vals of 2n states (ecap >= 2n) and a staging index of 2^lgs >= 2n slots;
 * the new table (ncap states) and its index (2^lgn slots); changed states (ccap) when asked. */
int tg_spw_step(int W, const void *keys, const void *vals, uint64_t n, uint64_t stride, const void *Hold, int lg_old,
                void *ekeys, void *evals, uint64_t ecap, void *Hs, int lgs, void *nkeys, void *nvals, uint64_t ncap,
                void *Hn, int lgn, void *ckeys, void *cvals, uint64_t ccap, const uint64_t *upd,
                const uint64_t *sel_mask, const uint64_t *sel_bits, int cap, int keep_below, int w, int want_changed,
                int use_h, int K, int ncls, const uint64_t *masks, const int64_t *weights, int64_t extra,
                const uint64_t *tmask, void *counters, void *stream);
/* the states with value < below (all for below < 0) into a new table with its index (truncate,
 * table from arrays); counters[0] = states written */
int tg_spw_filter(int W, const void *keys, const void *vals, uint64_t n, uint64_t stride, int below, void *nkeys,
                  void *nvals, uint64_t ncap, void *Hn, int lgn, void *counters, void *stream);
/* replaces sp_join (cdist/sparse_dp.c:207-236) for wide states: result (DEVICE uint64) =
 * min(total << 40 | changed state index), all ones when no pair meets */
int tg_spw_join(int W, const void *fkeys, const void *fvals, uint64_t nf, uint64_t fstride, const void *Hb, int lgb,
                const void *bkeys, uint64_t bstride, const uint64_t *tmask, void *result, void *stream);
/* values of m query keys (DEVICE uint64 [W][m]) in a table (255 = absent) */
int tg_spw_lookup(int W, const void *H, int lg, const void *keys, uint64_t stride, const void *q, uint64_t m,
                  void *out, void *stream);

/* A leg of column steps on wide states in one call, with the table sizes kept on the device and
 * one host read at the end (the multi-word counterpart of tg_sp_walk; the per-step rule of
 * cdist/sparse_dp.py:338-403).  steps HOST int64 [nsteps][13] = cap, keep_below, w, trunc (< 0:
 * none), keep (0, 1, 2: tables of at most 1024 states), join, ncls, use_h, extra, join table's keys
 * (DEVICE pointer), its index (DEVICE pointer), index bits, key stride; words HOST uint64
 * [nsteps][5][W] = upd, sel_mask, sel_bits, the bound's tmask, the join's tmask; masks HOST uint64
 * [nsteps][maxc][W], weights HOST int64 [nsteps][maxc].  scratch: tg_spw_walk_scratch_bytes(W,
 * cap, nsteps) DEVICE bytes, tables of at most cap states.  Kept tables go to the DEVICE arena: at
 * offset o, keys [W][s], vals [s] at o + 8 W s, index [2^lg] at o + 8 W s + round_up(s, 256).
 * out HOST int64 [nsteps][6] = states, changed states, kept offset (-1: not kept), kept stride s,
 * index bits, states before the cut's truncation; res HOST uint64 [nsteps][2 + W] = least join
 * total (all ones: none), forward value, forward key words.  Returns nsteps, or 0 with need[0]
 * (states per table) or need[1] (arena bytes) set: run the leg again with more room. */
int64_t tg_spw_walk_scratch_bytes(int W, uint64_t cap, int nsteps);
/* tables of at most limit / 2 states are stepped by one block per launch (default 512; 0: never);
 * returns the previous limit (a negative argument only reads it) */
int64_t tg_spw_set_small_limit(int64_t limit);
int tg_spw_walk(int W, int nsteps, const int64_t *steps, const uint64_t *words, const uint64_t *masks,
                const int64_t *weights, int maxc, int K, const void *keys0, const void *vals0, uint64_t n0,
                uint64_t stride0, void *scratch, uint64_t cap, void *arena, uint64_t arena_bytes, int64_t *out,
                uint64_t *res, int64_t *need, void *stream);

/* ---------------------------------------------------------------- completion tables (search)
 * Same entry points as the reference's ctypes binding (cdist/search.py:58-67): */
void *tg_tab_create(int log2slots, int wide, int *status);   /* cdist/gmitm.c:61 tab_create (NULL, *status -3: no memory) */
void tg_tab_free(void *t);                                    /* cdist/gmitm.c:78 tab_free */
int64_t tg_tab_count(void *t);                                /* cdist/gmitm.c:84 tab_count */
int64_t tg_tab_slots_log2(void *t);
/* cdist/gmitm.c:176 tab_build: zh, zl, lg are HOST uint64[n] */
int tg_tab_build(void *t, int n, const uint64_t *zh, const uint64_t *zl, const uint64_t *lg, int k);
/* batched form of cdist/gmitm.c:138 tab_lookup (static there): DEVICE arrays zh, zl, lg (uint64[m]),
 * R (int32[m]) -> out (int32[m]): least cost <= R[q] with the same fingerprint and another label, or -1 */
int tg_tab_lookup_dev(void *t, uint64_t m, const void *zh, const void *zl, const void *lg, const void *R,
                      void *out, void *stream);
/* A native probe for tg_search (no counterpart in the reference, whose DFS looks its table up in
 * the same process, cdist/gmitm.c:138-163): create it on a device table with room for `cap`
 * probes per round trip, pass tg_tab_probe as the probe and the handle as its context. */
void *tg_tab_probe_create(void *table, int64_t cap, int *status);
int tg_tab_probe(int64_t m, const uint64_t *zh, const uint64_t *zl, const uint64_t *lg, const int32_t *R,
                 int32_t *out, void *ctx);
void tg_tab_probe_free(void *ctx);
/* The reference's exact names and signatures, bound by cdist/search.py:58-67 (ctypes) and
 * defined at cdist/gmitm.c:61 (tab_create), :78 (tab_free), :84 (tab_count), :176 (tab_build):
 * thin forms of the tg_tab_* functions above (tab_create returns NULL on allocation failure). */
void *tab_create(int log2slots, int wide);
void tab_free(void *t);
int64_t tab_count(void *t);
void tab_build(void *t, int n, const uint64_t *zh, const uint64_t *zl, const uint64_t *lg, int k);

/* ---------------------------------------------------------------- batched dense Rank DP
 * Many plans (op streams ops[offsets[i]..offsets[i+1]), uint8) in one persistent launch fed from a
 * device work queue.  No counterpart in the reference, which runs one plan at a time
 * (cdist/auto.py:111-122).  info: arena bytes, jobs, units, plans.  values: HOST uint32[nplans]. */
void *tg_batch_create(int nplans, const int64_t *ops, const int64_t *offsets, int *status);
int tg_batch_info(void *batch, int64_t *info, int ninfo);
/* window: plans in progress at once (0: all), admitted widest first */
int tg_batch_run(void *batch, void *arena, int blocks, int window, uint32_t *values, void *stream);
void tg_batch_free(void *batch);
/* polls of one device wait for work before a block gives up and the run returns TG_ERR_TIMEOUT
 * (-5) with the context still usable; 0 restores the default (about 2.5 s of polling) */
int tg_batch_set_spin_limit(uint64_t polls);

/* ---------------------------------------------------------------- continuous serving
 * A long-lived persistent launch that takes new plans while it runs (no counterpart in the
 * reference, which solves one problem per process, cdist/__main__.py:64-108).  submit returns the
 * plan's slot or a negative status (-3: no room now; collect finished plans and retry); poll
 * returns finished (slot, final entry) pairs. */
void *tg_server_create(void *arena, uint64_t arena_bytes, int jcap, int64_t prm_bytes, int plan_cap, int blocks,
                       int *status);
int tg_server_submit(void *server, const int64_t *ops, int64_t nops);
/* the same for a plan scheduled ahead of time by tg_dense_plan (uint8); the handle stays the caller's */
int tg_server_submit_plan(void *server, void *plan);
int tg_server_poll(void *server, int *slots, uint32_t *values, int max);
int tg_server_stop(void *server);
void tg_server_free(void *server);

/* ---------------------------------------------------------------- weight-bounded search
 * One threshold K of the search for a minimum logical (the DFS of cdist/gmitm.c:597-740 with the
 * table probes collected into waves): columns as syndromes col[n][W], labels lg[n], table hashes
 * zh/zl[n]; rows -> columns CSR (row_start[nrows + 1], row_cols), columns -> rows (col_start[n + 1],
 * col_rows); rank[n] and the anchor columns in search order; kt the completion table's depth; probe
 * answers a wave of m probes (least cost <= R[i] with hash (zh, zl)[i] and a label other than lg[i],
 * or -1) and returns 0.  stats: nodes, lookups, hits, false hits, waves; sol / *nsol: the logical
 * found; ex_start / ex_cols (or NULL): each column's partners (f ^ y a column with their label),
 * forbidden below f; cover: the covering bound (0 off, 1 first dual, 2 with the ascent; stats[5] the
 * nodes it pruned); threads share out the anchors (the probe is entered by one at a time).  Returns 1 found, 0
 * exhausted, 2 time limit (seconds > 0), or a negative status. */
typedef int (*tg_probe_fn)(int64_t m, const uint64_t *zh, const uint64_t *zl, const uint64_t *lg, const int32_t *R,
                           int32_t *out, void *ctx);
int tg_search(int W, int n, int nrows, int wmax, const uint64_t *col, const uint64_t *lg, const uint64_t *zh,
              const uint64_t *zl, const int32_t *row_start, const int32_t *row_cols, const int32_t *col_start,
              const int32_t *col_rows, const int32_t *rank, const int32_t *anchors, int nanchors, int K, int kt,
              int64_t wave, tg_probe_fn probe, void *ctx, const int32_t *ex_start, const int32_t *ex_cols, int cover,
              int threads, double seconds, int64_t *stats, int32_t *sol, int32_t *nsol);

/* ---------------------------------------------------------------- tree DP (exact min-plus on a binary tree)
 * Per-call entry points with the reference's ctypes signatures (cdist/tree_dp.py:214-222), on DEVICE
 * tables: the pairs i in [start, stop) of a join in Gray order, out[parent] = min(out[parent], a + b)
 * over finite a, b (cdist/tree_dp.c:13-39); lm, rm are HOST arrays of `generators` (<= 64) maps. */
int tree_join_u8(const void *left, const void *right, void *out, const uint64_t *lm, const uint64_t *rm,
                 unsigned parent_bits, unsigned generators, uint64_t start, uint64_t stop, uint64_t infinity);
int tree_join_u16(const void *left, const void *right, void *out, const uint64_t *lm, const uint64_t *rm,
                  unsigned parent_bits, unsigned generators, uint64_t start, uint64_t stop, uint64_t infinity);
int tree_join_u32(const void *left, const void *right, void *out, const uint64_t *lm, const uint64_t *rm,
                  unsigned parent_bits, unsigned generators, uint64_t start, uint64_t stop, uint64_t infinity);
int tree_join_u64(const void *left, const void *right, void *out, const uint64_t *lm, const uint64_t *rm,
                  unsigned parent_bits, unsigned generators, uint64_t start, uint64_t stop, uint64_t infinity);
/* cdist/tree_dp.c:45-50 tree_move: memmove between DEVICE addresses */
int tree_move(void *destination, const void *source, size_t bytes);
/* Whole-tree plan (replaces the executor loop of cdist/tree_dp.py:442-501): uint32 tables in one
 * DEVICE arena.  leaves: rows (offset, size 1|2, column, nonzero); joins: rows (lo, ro, po, parent
 * rank, kernel generators, height >= 1, maps index, 0) in nondecreasing height; maps: uint32 (left,
 * right) state per generator.  info: heights, steps, launches per run, pairs, arena entries,
 * leaves, joins, single-block steps, block-product joins.  gemm: rows (join, F, mb, nb, kb, mapoff)
 * of joins run as min-plus products of 2^mb left and 2^nb right rows of 2^F entries (2^kb of them),
 * with their offset and parent vectors DL, DR, DT, PA, PB, PT (uint32) at gmaps[mapoff].
 * small_pairs (< 0: default): heights of at most that many pairs run in one single-block launch;
 * rbits (< 0: default): at most 2^rbits pairs per thread.  run: target = HOST bit vector of a
 * particular solution (ceil(ncols / 64) words); *value = root entry. */
void *tg_tree_plan(const int64_t *leaves, int64_t nleaves, const int64_t *joins, int64_t njoins,
                   const uint32_t *maps, int64_t nmaps, const int64_t *gemm, int64_t ngemm, const uint32_t *gmaps,
                   int64_t ngmaps, int64_t arena, int64_t root, int64_t ncols, int64_t small_pairs, int rbits,
                   int *status);
int tg_tree_plan_info(void *plan, int64_t *info, int n);
int tg_tree_run(void *plan, void *arena, const uint64_t *target, uint32_t inf, uint32_t *value, void *stream);
void tg_tree_plan_free(void *plan);

#ifdef __cplusplus
}
#endif
#endif
