// Weight-bounded search for a minimum logical with completion-table probes in waves (host code;
// the probes run on the device).  The search rules are the reference's (cdist/gmitm.c:597-740):
// every solution is searched from its lowest-rank column (the anchor; lower-rank columns are
// forbidden below it), a node branches on the columns of its unsatisfied row with the fewest free
// columns and excludes each branched column from the later siblings, and once the remaining budget
// fits the completion table (subsets of at most kt columns) the table decides.  Unlike the
// reference, which probes its table one node at a time, the probes of many nodes are collected into
// a wave (the children of every node one column above the table depth) and answered by one batched
// call, on the device in the package (csrc/table.cu); a hit is confirmed by an explicit search for
// the completion (a fingerprint collision is a false hit, as cdist/gmitm.c:636-650).
#include "tg_common.cuh"
#include "tg_capi.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace tg {

struct Search {
    int W, n, K, kt, wmax;
    const uint64_t *col, *lg, *zh, *zl;
    const int32_t *row_start, *row_cols, *col_start, *col_rows;
    const int32_t *ex_start = nullptr, *ex_cols = nullptr;   // partners: f ^ y is a column with f's and y's label
    std::vector<uint8_t> forb;             // 0 free, else the stamp that forbade the column
    std::vector<int> avail;                // free columns per row
    std::vector<uint64_t> syn;             // per depth: W words
    std::vector<uint64_t> g, hz, lz;       // per depth: label, hashes
    std::vector<int> path;
    // the wave of probes: hashes, label, budget; and what each probe stands for (a node's path,
    // plus one child column or -1)
    std::vector<uint64_t> pzh, pzl, plg;
    std::vector<int32_t> pR, pnode, pchild, pout;
    std::vector<int32_t> store;            // node paths, flattened
    std::vector<int64_t> node_off;
    std::vector<int32_t> node_len;
    int64_t wave;
    tg_probe_fn probe;
    void *ctx;
    bool found = false, timeout = false, failed = false;
    std::atomic<int> *stop = nullptr;     // shared by the threads of one search: set when one stops
    std::mutex *mu = nullptr;             // one wave at a time through the probe
    bool halted() const { return found || timeout || failed || (stop && stop->load(std::memory_order_relaxed)); }
    std::vector<int> sol;
    int64_t nodes = 0, lookups = 0, hits = 0, false_hits = 0, waves = 0;
    std::chrono::steady_clock::time_point deadline;
    bool limited = false;

    uint64_t *S(int d) { return syn.data() + (size_t)d * W; }
    int pop(const uint64_t *s) const {
        int c = 0;
        for (int w = 0; w < W; w++) c += __builtin_popcountll(s[w]);
        return c;
    }
    void forbid(int f, uint8_t stamp) {
        if (forb[f]) return;
        forb[f] = stamp;
        for (int q = col_start[f]; q < col_start[f + 1]; q++) avail[col_rows[q]]--;
    }
    void unforbid(int f) {
        if (!forb[f]) return;
        forb[f] = 0;
        for (int q = col_start[f]; q < col_start[f + 1]; q++) avail[col_rows[q]]++;
    }
    // covering bound (cdist/gmitm.c:496-596): each unsatisfied row needs a free column; the weights
    // y_r = 1 / (most unsatisfied rows one free column of r clears) are a feasible dual of the covering
    // LP, raised greedily (rows with the fewest free columns first) while every column's load stays
    // <= 1; their sum bounds the columns still needed from below.  Returns true to prune.
    int cover = 0;                                    // 0 off, 1 the first dual only, 2 with the ascent
    std::vector<double> load;
    std::vector<int> cv_rows;
    std::vector<double> cv_y;
    int64_t cover_pruned = 0;
    bool cover_prune(const uint64_t *s, int R, int pc) {
        const double lim = R + 1e-9, inv_wmax = 1.0 / wmax;
        int left = pc;
        if (left * inv_wmax > lim) return true;
        double sum = 0.0;
        cv_rows.clear();
        cv_y.clear();
        for (int w = 0; w < W; w++) {
            uint64_t x = s[w];
            while (x) {
                const int r = w * 64 + __builtin_ctzll(x);
                x &= x - 1;
                left--;
                int m = 0;
                for (int q = row_start[r]; q < row_start[r + 1]; q++) {
                    const int f = row_cols[q];
                    if (forb[(size_t)f]) continue;
                    int o = 0;
                    for (int v = 0; v < W; v++) o += __builtin_popcountll(s[v] & col[(size_t)f * W + v]);
                    m = std::max(m, o);
                }
                if (m == 0) return true;              // no free column reaches this row
                sum += 1.0 / m;
                if (sum + left * inv_wmax > lim) return true;
                if (cover < 2) {
                    // first dual only: once even weight 1 on every remaining row cannot pass the
                    // budget, this node is not pruned (the rows left need not be scanned)
                    if (sum + left <= lim) return false;
                    continue;
                }
                cv_rows.push_back(r);
                cv_y.push_back(1.0 / m);
            }
        }
        if (cover < 2) return false;
        if (load.size() != (size_t)n) load.assign((size_t)n, 0.0);
        for (size_t i = 0; i < cv_rows.size(); i++)
            for (int q = row_start[cv_rows[i]]; q < row_start[cv_rows[i] + 1]; q++) load[(size_t)row_cols[q]] = 0.0;
        for (size_t i = 0; i < cv_rows.size(); i++)
            for (int q = row_start[cv_rows[i]]; q < row_start[cv_rows[i] + 1]; q++)
                if (!forb[(size_t)row_cols[q]]) load[(size_t)row_cols[q]] += cv_y[i];
        std::vector<int> ord(cv_rows.size());
        for (size_t i = 0; i < ord.size(); i++) ord[i] = (int)i;
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return avail[(size_t)cv_rows[(size_t)a]] <
                                                                           avail[(size_t)cv_rows[(size_t)b]]; });
        for (int i : ord) {
            const int r = cv_rows[(size_t)i];
            double slack = 1.0;
            for (int q = row_start[r]; q < row_start[r + 1]; q++)
                if (!forb[(size_t)row_cols[q]]) slack = std::min(slack, 1.0 - load[(size_t)row_cols[q]]);
            if (slack <= 1e-12) continue;
            for (int q = row_start[r]; q < row_start[r + 1]; q++)
                if (!forb[(size_t)row_cols[q]]) load[(size_t)row_cols[q]] += slack;
            sum += slack;
            if (sum > lim) return true;
        }
        return false;
    }

    // a minimum logical holding f holds none of f's partners: forbid them below f (undone by the caller)
    static constexpr uint8_t PARTNER = 253;
    void exclude(int f, std::vector<int> &undo) {
        if (!ex_start) return;
        for (int q = ex_start[f]; q < ex_start[f + 1]; q++) {
            const int y = ex_cols[q];
            if (!forb[(size_t)y]) { forbid(y, PARTNER); undo.push_back(y); }
        }
    }
    void push(int d, int f) {          // state d + 1 = state d with column f
        const uint64_t *a = S(d);
        uint64_t *b = S(d + 1);
        const uint64_t *c = col + (size_t)f * W;
        for (int w = 0; w < W; w++) b[w] = a[w] ^ c[w];
        g[d + 1] = g[d] ^ lg[f];
        hz[d + 1] = hz[d] ^ zh[f];
        lz[d + 1] = lz[d] ^ zl[f];
        path[d] = f;
    }
    int node_here(int d) {
        node_off.push_back((int64_t)store.size());
        node_len.push_back(d);
        store.insert(store.end(), path.begin(), path.begin() + d);
        return (int)node_off.size() - 1;
    }
    void add_probe(uint64_t h, uint64_t l, uint64_t lab, int R, int node, int child) {
        pzh.push_back(h); pzl.push_back(l); plg.push_back(lab); pR.push_back(R);
        pnode.push_back(node); pchild.push_back(child);
        lookups++;
    }
    // a wave is sent only between nodes (a node's probes refer to its stored path)
    void room(int64_t more) {
        if ((int64_t)pzh.size() + more > wave) flush();
    }
    // T with |T| <= budget, syndrome s and a label other than lab (S xor T is then a logical); a
    // column tried at a level is excluded from that level's later branches (stamp = level + 1)
    bool complete(std::vector<uint64_t> &s, uint64_t lab, int budget, int level, std::vector<int> &T,
                  std::vector<int> &used) {
        const int pc = pop(s.data());
        if (pc == 0) return lab != 0;
        if (budget <= 0 || pc > wmax * budget) return false;
        int piv = -1;
        for (int w = 0; w < W && piv < 0; w++)
            if (s[(size_t)w]) piv = w * 64 + __builtin_ctzll(s[(size_t)w]);
        bool ok = false;
        for (int q = row_start[piv]; q < row_start[piv + 1] && !ok; q++) {
            const int f = row_cols[q];
            if (used[(size_t)f]) continue;
            used[(size_t)f] = level + 1;
            for (int w = 0; w < W; w++) s[(size_t)w] ^= col[(size_t)f * W + w];
            T.push_back(f);
            ok = complete(s, lab ^ lg[f], budget - 1, level + 1, T, used);
            if (!ok) T.pop_back();
            for (int w = 0; w < W; w++) s[(size_t)w] ^= col[(size_t)f * W + w];
        }
        for (int q = row_start[piv]; q < row_start[piv + 1]; q++)
            if (used[(size_t)row_cols[q]] == level + 1) used[(size_t)row_cols[q]] = 0;
        return ok;
    }
    void flush() {
        const int64_t m = (int64_t)pzh.size();
        if (!m) return;
        waves++;
        pout.assign((size_t)m, -1);
        {
            std::unique_lock<std::mutex> lock;
            if (mu) lock = std::unique_lock<std::mutex>(*mu);
            if (probe(m, pzh.data(), pzl.data(), plg.data(), pR.data(), pout.data(), ctx) != 0) failed = true;
        }
        if (limited && std::chrono::steady_clock::now() > deadline) timeout = true;
        for (int64_t i = 0; i < m && !found && !failed; i++) {
            if (pout[(size_t)i] < 0) continue;
            hits++;
            // the probe's state: its node's path plus its child
            std::vector<int> Sx(store.begin() + node_off[(size_t)pnode[(size_t)i]],
                                store.begin() + node_off[(size_t)pnode[(size_t)i]] + node_len[(size_t)pnode[(size_t)i]]);
            if (pchild[(size_t)i] >= 0) Sx.push_back(pchild[(size_t)i]);
            std::vector<uint64_t> s((size_t)W, 0);
            uint64_t lab = 0;
            for (int f : Sx) {
                for (int w = 0; w < W; w++) s[(size_t)w] ^= col[(size_t)f * W + w];
                lab ^= lg[f];
            }
            std::vector<int> T;
            std::vector<int> used((size_t)n, 0);
            if (complete(s, lab, pR[(size_t)i], 0, T, used)) {
                // the logical is the symmetric difference of the prefix and the completion
                std::vector<int> X = Sx;
                for (int f : T) {
                    auto it = std::find(X.begin(), X.end(), f);
                    if (it != X.end()) X.erase(it); else X.push_back(f);
                }
                std::sort(X.begin(), X.end());
                sol = X;
                found = true;
            } else {
                false_hits++;
            }
        }
        pzh.clear(); pzl.clear(); plg.clear(); pR.clear(); pnode.clear(); pchild.clear();
        store.clear(); node_off.clear(); node_len.clear();
    }
    void dfs(int d) {
        if (halted()) return;
        nodes++;
        if (limited && (nodes & 4095) == 0 && std::chrono::steady_clock::now() > deadline) { timeout = true; return; }
        const uint64_t *s = S(d);
        const int pc = pop(s);
        if (pc == 0) {
            if (g[d] != 0) { sol.assign(path.begin(), path.begin() + d); std::sort(sol.begin(), sol.end()); found = true; }
            return;
        }
        const int R = K - d;
        if (R <= 0 || pc > wmax * R) return;
        if (R <= kt) {                                   // the table decides this node
            room(1);
            if (found || failed) return;
            add_probe(hz[d], lz[d], g[d], R, node_here(d), -1);
            return;
        }
        // the covering bound on nodes beyond the table's reach (R > kt here) with more unsatisfied
        // rows than budget, the gate of cdist/gmitm.c:610 at its default factor
        if (cover && pc > R && cover_prune(s, R, pc)) {
            cover_pruned++;
            return;
        }
        int piv = -1, best = 1 << 30;
        for (int w = 0; w < W; w++) {
            uint64_t x = s[w];
            while (x) {
                const int r = w * 64 + __builtin_ctzll(x);
                x &= x - 1;
                if (avail[r] < best) { best = avail[r]; piv = r; }
            }
        }
        if (best == 0) return;
        const uint8_t stamp = (uint8_t)(d + 1);
        if (R - 1 <= kt) {
            // every child is decided by one probe: no bookkeeping below this node
            room(row_start[piv + 1] - row_start[piv]);
            if (found || failed) return;
            const int node = node_here(d);
            for (int q = row_start[piv]; q < row_start[piv + 1]; q++) {
                const int f = row_cols[q];
                if (forb[f]) continue;
                forbid(f, stamp);
                const uint64_t *c = col + (size_t)f * W;
                bool zero = true;
                for (int w = 0; w < W && zero; w++) zero = (s[w] ^ c[w]) == 0;
                nodes++;
                if (zero) {
                    if ((g[d] ^ lg[f]) != 0) {
                        sol.assign(path.begin(), path.begin() + d);
                        sol.push_back(f);
                        std::sort(sol.begin(), sol.end());
                        found = true;
                        break;
                    }
                    continue;
                }
                add_probe(hz[d] ^ zh[f], lz[d] ^ zl[f], g[d] ^ lg[f], R - 1, node, f);
            }
        } else {
            std::vector<int> undo;
            for (int q = row_start[piv]; q < row_start[piv + 1]; q++) {
                const int f = row_cols[q];
                if (forb[f]) continue;
                forbid(f, stamp);
                push(d, f);
                undo.clear();
                exclude(f, undo);
                dfs(d + 1);
                for (int y : undo) unforbid(y);
                if (halted()) break;
            }
        }
        for (int q = row_start[piv]; q < row_start[piv + 1]; q++)
            if (forb[row_cols[q]] == stamp) unforbid(row_cols[q]);
    }
};

}  // namespace tg

using namespace tg;

extern "C" {

// One threshold K: is there a logical (zero syndrome, label != 0) of at most K columns?  Columns:
// syndromes col[n][W] (uint64 words), labels lg[n], table hashes zh/zl[n]; rows -> columns CSR
// (row_start[nrows + 1], row_cols) and columns -> rows (col_start[n + 1], col_rows); rank[n] (the
// anchor of a solution is its lowest-rank column), anchors: the columns to start from, in order;
// kt: the completion table holds every subset of at most kt columns; probe(m, zh, zl, lg, R, out,
// ctx) answers a wave of probes (least cost <= R with the same hash and another label, or -1).
// stats: nodes, lookups, hits, false hits, waves.  sol: the logical's columns (sorted), *nsol its
// size; ex_start / ex_cols (or NULL): each column's partners (columns y with f ^ y equal to a column of
// the same label: a minimum logical never holds both; cdist/search.py:207-231), forbidden below f;
// cover: the covering bound (0 off, 1 its first dual, 2 with the ascent); stats[5]: nodes it pruned;
// threads: threads sharing out the anchors (the probe is entered by one at a time).  Returns 1
// found, 0 exhausted, 2 time limit, or a negative status (-6: the probe call failed).
int tg_search(int W, int n, int nrows, int wmax, const uint64_t *col, const uint64_t *lg, const uint64_t *zh,
              const uint64_t *zl, const int32_t *row_start, const int32_t *row_cols, const int32_t *col_start,
              const int32_t *col_rows, const int32_t *rank, const int32_t *anchors, int nanchors, int K, int kt,
              int64_t wave, tg_probe_fn probe, void *ctx, const int32_t *ex_start, const int32_t *ex_cols, int cover,
              int threads, double seconds, int64_t *stats, int32_t *sol, int32_t *nsol) {
    if (W < 1 || n < 0 || nrows < 0 || K < 1 || K > 64 || kt < 0 || !col || !lg || !zh || !zl || !row_start ||
        !col_start || !rank || (nanchors && !anchors) || !probe || !stats || !sol || !nsol || wave < 1)
        return set_error(TG_ERR_ARG, "bad search arguments");
    for (int a = 0; a < nanchors; a++)
        if (anchors[a] < 0 || anchors[a] >= n) return set_error(TG_ERR_ARG, "anchor out of range");
    const int T = std::max(1, std::min(threads, std::max(1, nanchors)));
    std::atomic<int> stop(0), next(0);
    std::mutex mu;
    std::vector<Search> Xs((size_t)T);
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::microseconds((int64_t)(seconds * 1e6));
    for (Search &X : Xs) {
        X.W = W; X.n = n; X.K = K; X.kt = kt; X.wmax = std::max(1, wmax);
        X.col = col; X.lg = lg; X.zh = zh; X.zl = zl;
        X.row_start = row_start; X.row_cols = row_cols; X.col_start = col_start; X.col_rows = col_rows;
        X.forb.assign((size_t)n, 0);
        X.avail.assign((size_t)nrows, 0);
        X.syn.assign((size_t)(K + 2) * W, 0);
        X.g.assign((size_t)K + 2, 0); X.hz.assign((size_t)K + 2, 0); X.lz.assign((size_t)K + 2, 0);
        X.path.assign((size_t)K + 2, -1);
        X.wave = wave; X.probe = probe; X.ctx = ctx;
        X.limited = seconds > 0;
        X.deadline = deadline;
        X.stop = &stop;
        X.mu = &mu;
        X.ex_start = ex_start;
        X.ex_cols = ex_cols;
        X.cover = std::max(0, std::min(cover, 2));
    }
    // anchors are handed out one at a time; each thread searches below its anchors with its own
    // forbidden set and wave
    auto work = [&](Search &X) {
        while (!X.halted()) {
            const int a = next.fetch_add(1);
            if (a >= nanchors) break;
            const int f0 = anchors[a];
            for (int r = 0; r < nrows; r++) X.avail[(size_t)r] = row_start[r + 1] - row_start[r];
            std::fill(X.forb.begin(), X.forb.end(), 0);
            for (int f = 0; f < n; f++)
                if (rank[f] < rank[f0]) X.forbid(f, 255);
            X.forbid(f0, 254);
            X.push(0, f0);
            std::vector<int> undo;
            X.exclude(f0, undo);
            X.dfs(1);
        }
        if (!X.halted()) X.flush();
        if (X.found || X.timeout || X.failed) stop.store(1);
    };
    if (T == 1) {
        work(Xs[0]);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < T; t++) pool.emplace_back(work, std::ref(Xs[(size_t)t]));
        for (auto &th : pool) th.join();
    }
    int64_t tot[6] = {0, 0, 0, 0, 0, 0};
    bool any_timeout = false, any_failed = false;
    const Search *hit = nullptr;
    for (const Search &X : Xs) {
        tot[0] += X.nodes; tot[1] += X.lookups; tot[2] += X.hits; tot[3] += X.false_hits; tot[4] += X.waves;
        tot[5] += X.cover_pruned;
        any_timeout |= X.timeout;
        any_failed |= X.failed;
        if (X.found && !hit) hit = &X;
    }
    for (int i = 0; i < 6; i++) stats[i] = tot[i];
    *nsol = 0;
    if (hit) {
        for (size_t i = 0; i < hit->sol.size() && i < 64; i++) sol[i] = hit->sol[i];
        *nsol = (int32_t)hit->sol.size();
        return 1;
    }
    if (any_failed) return set_error(TG_ERR_STATE, "the probe call failed");
    return any_timeout ? 2 : 0;
}

}  // extern "C"
