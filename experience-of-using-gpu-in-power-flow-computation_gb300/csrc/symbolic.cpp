// symbolic.cpp -- once-per-topology analysis on the host: Ybus pattern and
// assembly map, fill-reducing ordering of the buses, symbolic block LU of the
// Newton Jacobian, its Crout gather lists and level schedules, and the map
// from factor block positions to Ybus slots used by the Jacobian fill.
#include <algorithm>
#include <numeric>
#include <queue>
#include <string>
#include <vector>

#include "gbpf_internal.h"

namespace gbpf {

int YPattern::find(int r, int c) const {
    auto b = col.begin() + rowptr[r], e = col.begin() + rowptr[r + 1];
    auto it = std::lower_bound(b, e, c);
    return (it != e && *it == c) ? (int)(it - col.begin()) : -1;
}

// Pattern of calcYbusSp_eficinte (GPU/sistema.h:705-758): four stamps per
// branch and one shunt per bus, duplicates summed.  Slot contributions are
// listed in the order Eigen's setFromTriplets adds them: the stamps of branch
// 0 (de,para), (para,de), (de,de), (para,para), then branch 1, ..., then the
// bus shunts.
YPattern build_ypattern(const Grid &g) {
    YPattern y;
    const int n = g.nB;
    y.n = n;
    std::vector<std::vector<int>> rows(n);
    for (int k = 0; k < n; k++) rows[k].push_back(k);
    for (int b = 0; b < g.nL; b++) {
        const int f = g.de[b] - 1, t = g.para[b] - 1;
        rows[f].push_back(t);
        rows[t].push_back(f);
    }
    y.rowptr.assign(n + 1, 0);
    for (int k = 0; k < n; k++) {
        auto &r = rows[k];
        std::sort(r.begin(), r.end());
        r.erase(std::unique(r.begin(), r.end()), r.end());
        y.rowptr[k + 1] = y.rowptr[k] + (int)r.size();
    }
    y.nnz = y.rowptr[n];
    y.col.resize(y.nnz);
    for (int k = 0; k < n; k++) std::copy(rows[k].begin(), rows[k].end(), y.col.begin() + y.rowptr[k]);
    y.diag.resize(n);
    for (int k = 0; k < n; k++) y.diag[k] = y.find(k, k);
    // contributions in triplet order
    std::vector<int> cnt(y.nnz, 0);
    std::vector<std::pair<int, int>> trip;  // (slot, source)
    trip.reserve(4 * g.nL + n);
    for (int b = 0; b < g.nL; b++) {
        const int f = g.de[b] - 1, t = g.para[b] - 1;
        trip.push_back({y.find(f, t), 4 * b + 0});
        trip.push_back({y.find(t, f), 4 * b + 1});
        trip.push_back({y.find(f, f), 4 * b + 2});
        trip.push_back({y.find(t, t), 4 * b + 3});
    }
    for (int k = 0; k < n; k++) trip.push_back({y.diag[k], -1 - k});
    for (auto &p : trip) cnt[p.first]++;
    y.cptr.assign(y.nnz + 1, 0);
    for (int s = 0; s < y.nnz; s++) y.cptr[s + 1] = y.cptr[s] + cnt[s];
    y.csrc.resize(trip.size());
    std::vector<int> fill(y.cptr.begin(), y.cptr.end() - 1);
    for (auto &p : trip) y.csrc[fill[p.first]++] = p.second;
    return y;
}

// Minimum degree on an explicit elimination graph (ties broken by the lower
// index), giving the order in which blocks are eliminated.
std::vector<int> min_degree_order(int n, const std::vector<std::vector<int>> &adj0) {
    std::vector<std::vector<int>> adj(adj0);
    std::vector<int> deg(n), mark(n, 0), done(n, 0), order;
    order.reserve(n);
    int stamp = 0;
    using E = std::pair<int, int>;
    std::priority_queue<E, std::vector<E>, std::greater<E>> pq;
    for (int i = 0; i < n; i++) { deg[i] = (int)adj[i].size(); pq.push({deg[i], i}); }
    std::vector<int> nb, tmp;
    while ((int)order.size() < n) {
        E e = pq.top();
        pq.pop();
        const int p = e.second;
        if (done[p] || e.first != deg[p]) continue;
        done[p] = 1;
        order.push_back(p);
        nb.clear();
        for (int v : adj[p]) if (!done[v]) nb.push_back(v);
        for (int u : nb) {
            ++stamp;
            mark[u] = stamp;
            tmp.clear();
            for (int v : adj[u]) if (v != p && !done[v] && mark[v] != stamp) { mark[v] = stamp; tmp.push_back(v); }
            for (int v : nb) if (mark[v] != stamp) { mark[v] = stamp; tmp.push_back(v); }
            adj[u] = tmp;
            deg[u] = (int)tmp.size();
            pq.push({deg[u], u});
        }
        adj[p].clear();
        adj[p].shrink_to_fit();
    }
    return order;
}

// Shorter elimination tree at no extra fill (Jess and Kees, "A data structure
// for parallel L/U decomposition", IEEE Trans. Computers C-31, 1982): the
// filled graph of `ord` is chordal, and eliminating, round after round, a
// maximal independent set of its simplicial vertices (neighbourhood a clique)
// is a perfect elimination order of it -- no fill beyond that of `ord` -- whose
// elimination tree is as short as such an order allows.  Every round becomes
// one level of the factor's schedule, and each level costs the Newton kernels a
// barrier and a chain of dependent 2x2 products, so fewer levels is less
// latency per iteration (118-bus grid: 30 -> 21 levels, same factor).
// Within a round the vertices keep their order in `ord`.
std::vector<int> reduce_height(int n, const std::vector<std::vector<int>> &adj, const std::vector<int> &ord) {
    std::vector<int> pos(n);
    for (int i = 0; i < n; i++) pos[ord[i]] = i;
    // filled graph: elimination of ord on a copy of the graph (sorted adjacency)
    std::vector<std::vector<int>> F(n);
    {
        std::vector<std::vector<int>> up(n);  // higher neighbours, by position
        for (int v = 0; v < n; v++)
            for (int w : adj[v]) if (pos[w] > pos[v]) up[v].push_back(w);
        std::vector<int> mark(n, -1);
        for (int i = 0; i < n; i++) {
            const int v = ord[i];
            auto &u = up[v];
            std::sort(u.begin(), u.end(), [&](int a, int b) { return pos[a] < pos[b]; });
            u.erase(std::unique(u.begin(), u.end()), u.end());
            for (int w : u) { F[v].push_back(w); F[w].push_back(v); }
            if (u.empty()) continue;
            // the lowest higher neighbour inherits the rest (elimination-tree parent)
            const int p = u[0];
            auto &pu = up[p];
            for (size_t k = 1; k < u.size(); k++) pu.push_back(u[k]);
            (void)mark;
        }
        for (auto &f : F) {
            std::sort(f.begin(), f.end());
            f.erase(std::unique(f.begin(), f.end()), f.end());
        }
    }
    std::vector<char> alive(n, 1), simp(n, 0), dirty(n, 1);
    std::vector<int> deg(n);
    for (int v = 0; v < n; v++) deg[v] = (int)F[v].size();
    auto adjacent = [&](int a, int b) { return std::binary_search(F[a].begin(), F[a].end(), b); };
    auto simplicial = [&](int v) {
        std::vector<int> nb;
        for (int w : F[v]) if (alive[w]) nb.push_back(w);
        for (size_t x = 0; x < nb.size(); x++)
            for (size_t z = x + 1; z < nb.size(); z++)
                if (!adjacent(nb[x], nb[z])) return false;
        return true;
    };
    std::vector<int> out, cand, blocked(n, -1);
    out.reserve(n);
    int left = n, round = 0;
    while (left > 0) {
        cand.clear();
        for (int i = 0; i < n; i++) {
            const int v = ord[i];
            if (!alive[v]) continue;
            if (dirty[v]) { simp[v] = simplicial(v); dirty[v] = 0; }
            if (simp[v]) cand.push_back(v);
        }
        // maximal independent set, lowest degree first, ties in ord order
        std::stable_sort(cand.begin(), cand.end(), [&](int a, int b) { return deg[a] < deg[b]; });
        std::vector<int> chosen;
        for (int v : cand) {
            if (blocked[v] == round) continue;
            chosen.push_back(v);
            blocked[v] = round;
            for (int w : F[v]) if (alive[w]) blocked[w] = round;
        }
        std::sort(chosen.begin(), chosen.end(), [&](int a, int b) { return pos[a] < pos[b]; });
        for (int v : chosen) {
            alive[v] = 0;
            left--;
            out.push_back(v);
            for (int w : F[v]) if (alive[w]) { dirty[w] = 1; deg[w]--; }
        }
        round++;
    }
    return out;
}

Symbolic analyse(const Grid &g, const YPattern &y, std::string *why) {
    Symbolic S;
    const int nB = g.nB, s = g.slack - 1, n = nB - 1;
    S.n = n;
    // bus graph without the slack
    std::vector<int> cidx(nB, -1), cbus;
    for (int k = 0; k < nB; k++) if (k != s) { cidx[k] = (int)cbus.size(); cbus.push_back(k); }
    std::vector<std::vector<int>> adj(n);
    for (int k = 0; k < nB; k++) {
        if (k == s) continue;
        for (int p = y.rowptr[k]; p < y.rowptr[k + 1]; p++) {
            const int m = y.col[p];
            if (m == s || m == k) continue;
            adj[cidx[k]].push_back(cidx[m]);
        }
    }
    std::vector<int> ord = reduce_height(n, adj, min_degree_order(n, adj));
    S.bus_of_blk.resize(n);
    S.blk_of_bus.assign(nB, -1);
    for (int b = 0; b < n; b++) {
        S.bus_of_blk[b] = cbus[ord[b]];
        S.blk_of_bus[cbus[ord[b]]] = b;
    }
    // lower structure of A in the new order: for column j, rows i > j
    std::vector<std::vector<int>> alow(n);
    for (int k = 0; k < nB; k++) {
        if (k == s) continue;
        const int bk = S.blk_of_bus[k];
        for (int p = y.rowptr[k]; p < y.rowptr[k + 1]; p++) {
            const int m = y.col[p];
            if (m == s || m == k) continue;
            const int bm = S.blk_of_bus[m];
            if (bm > bk) alow[bk].push_back(bm);
        }
    }
    // symbolic factorisation: struct(j) = alow(j) U (struct(c) \ {j}) over the
    // elimination-tree children c of j
    std::vector<std::vector<int>> st(n), children(n);
    std::vector<int> mark(n, -1);
    for (int j = 0; j < n; j++) {
        std::vector<int> &out = st[j];
        mark[j] = j;
        for (int i : alow[j]) if (mark[i] != j) { mark[i] = j; out.push_back(i); }
        for (int c : children[j])
            for (int i : st[c]) if (i != j && mark[i] != j) { mark[i] = j; out.push_back(i); }
        std::sort(out.begin(), out.end());
        if (!out.empty()) children[out[0]].push_back(j);
    }
    S.up_ptr.assign(n + 1, 0);
    for (int j = 0; j < n; j++) S.up_ptr[j + 1] = S.up_ptr[j] + (int)st[j].size();
    S.nup = S.up_ptr[n];
    S.up_col.resize(S.nup);
    for (int j = 0; j < n; j++) std::copy(st[j].begin(), st[j].end(), S.up_col.begin() + S.up_ptr[j]);
    auto pos_in = [&](int j, int i) -> int {
        auto b = S.up_col.begin() + S.up_ptr[j], e = S.up_col.begin() + S.up_ptr[j + 1];
        auto it = std::lower_bound(b, e, i);
        return (it != e && *it == i) ? (int)(it - S.up_col.begin()) : -1;
    };
    // row structures rs(j) = {k : j in idx(k)}, k ascending, with positions
    std::vector<int> rcnt(n, 0);
    for (int p = 0; p < S.nup; p++) rcnt[S.up_col[p]]++;
    S.dg_ptr.assign(n + 1, 0);
    for (int j = 0; j < n; j++) S.dg_ptr[j + 1] = S.dg_ptr[j] + rcnt[j];
    S.dg_pos.resize(S.nup);
    S.dg_k.resize(S.nup);
    {
        std::vector<int> f(S.dg_ptr.begin(), S.dg_ptr.end() - 1);
        for (int k = 0; k < n; k++)
            for (int p = S.up_ptr[k]; p < S.up_ptr[k + 1]; p++) {
                const int j = S.up_col[p];
                S.dg_pos[f[j]] = p;
                S.dg_k[f[j]] = k;
                f[j]++;
            }
    }
    // off-diagonal gather pairs: for k, a < b in idx(k): entry (j = idx(k)[a], i = idx(k)[b])
    std::vector<long long> ocnt(S.nup, 0);
    for (int k = 0; k < n; k++)
        for (int a = S.up_ptr[k]; a < S.up_ptr[k + 1]; a++)
            for (int b = a + 1; b < S.up_ptr[k + 1]; b++) {
                const int p = pos_in(S.up_col[a], S.up_col[b]);
                if (p < 0) { if (why) *why = "symbolic factorisation is not closed under fill"; return Symbolic(); }
                ocnt[p]++;
            }
    S.og_ptr.assign(S.nup + 1, 0);
    for (int p = 0; p < S.nup; p++) S.og_ptr[p + 1] = S.og_ptr[p] + ocnt[p];
    const long long npairs = S.og_ptr[S.nup];
    S.og_a.resize(npairs);
    S.og_b.resize(npairs);
    S.og_k.resize(npairs);
    {
        std::vector<long long> f(S.og_ptr.begin(), S.og_ptr.end() - 1);
        for (int k = 0; k < n; k++)
            for (int a = S.up_ptr[k]; a < S.up_ptr[k + 1]; a++)
                for (int b = a + 1; b < S.up_ptr[k + 1]; b++) {
                    const int p = pos_in(S.up_col[a], S.up_col[b]);
                    S.og_a[f[p]] = a;
                    S.og_b[f[p]] = b;
                    S.og_k[f[p]] = k;
                    f[p]++;
                }
    }
    // level schedules
    std::vector<int> fl(n, 0), bl(n, 0);
    int nfl = 0, nbl = 0;
    for (int j = 0; j < n; j++) {
        int l = 0;
        for (int q = S.dg_ptr[j]; q < S.dg_ptr[j + 1]; q++) l = std::max(l, fl[S.dg_k[q]] + 1);
        fl[j] = l;
        nfl = std::max(nfl, l + 1);
    }
    for (int j = n - 1; j >= 0; j--) {
        int l = 0;
        for (int p = S.up_ptr[j]; p < S.up_ptr[j + 1]; p++) l = std::max(l, bl[S.up_col[p]] + 1);
        bl[j] = l;
        nbl = std::max(nbl, l + 1);
    }
    auto bucket = [n](const std::vector<int> &lev, int nl, std::vector<int> &ptr, std::vector<int> &steps) {
        ptr.assign(nl + 1, 0);
        for (int j = 0; j < n; j++) ptr[lev[j] + 1]++;
        for (int l = 0; l < nl; l++) ptr[l + 1] += ptr[l];
        steps.resize(n);
        std::vector<int> f(ptr.begin(), ptr.end() - 1);
        for (int j = 0; j < n; j++) steps[f[lev[j]]++] = j;
    };
    bucket(fl, nfl, S.flev_ptr, S.flev_steps);
    bucket(bl, nbl, S.blev_ptr, S.blev_steps);
    S.fent_ptr.assign(nfl + 1, 0);
    S.fent_p.clear();
    S.fent_j.clear();
    for (int l = 0; l < nfl; l++) {
        for (int t = S.flev_ptr[l]; t < S.flev_ptr[l + 1]; t++) {
            const int j = S.flev_steps[t];
            for (int p = S.up_ptr[j]; p < S.up_ptr[j + 1]; p++) { S.fent_p.push_back(p); S.fent_j.push_back(j); }
        }
        S.fent_ptr[l + 1] = (int)S.fent_p.size();
    }
    // Jacobian fill map over factor block positions
    const int nq = n + 2 * S.nup;
    S.ysl.resize(nq);
    S.rbus.resize(nq);
    S.cbus.resize(nq);
    for (int j = 0; j < n; j++) {
        const int bj = S.bus_of_blk[j];
        S.ysl[j] = y.diag[bj];
        S.rbus[j] = bj;
        S.cbus[j] = bj;
    }
    for (int j = 0; j < n; j++)
        for (int p = S.up_ptr[j]; p < S.up_ptr[j + 1]; p++) {
            const int bi = S.bus_of_blk[S.up_col[p]], bj = S.bus_of_blk[j];
            const int ql = n + p, qu = n + S.nup + p;
            S.ysl[ql] = y.find(bi, bj);  // L(i,j): row bus i, column bus j
            S.rbus[ql] = bi;
            S.cbus[ql] = bj;
            S.ysl[qu] = y.find(bj, bi);  // U(j,i): row bus j, column bus i
            S.rbus[qu] = bj;
            S.cbus[qu] = bi;
        }
    return S;
}

}  // namespace gbpf

extern "C" gbpf_status gbpf_grid_analyse(const gbpf_grid *h, long long info[8]) {
    if (!h || !info) return GBPF_E_ARG;
    const gbpf::Grid &g = h->g;
    if (g.nB < 2 || g.slack < 1) return GBPF_E_INPUT;
    const gbpf::YPattern y = gbpf::build_ypattern(g);
    std::string why;
    const gbpf::Symbolic S = gbpf::analyse(g, y, &why);
    if (S.n != g.nB - 1) {
        gbpf::set_error("symbolic analysis failed: " + why);
        return GBPF_E_INPUT;
    }
    long long jblocks = 0;
    for (int q = 0; q < S.n + 2 * S.nup; q++) jblocks += S.ysl[q] >= 0;
    // closure: every pair target (a, b) of entry p lies in an earlier step's row
    bool closed = true;
    for (int j = 0; j < S.n && closed; j++)
        for (int p = S.up_ptr[j]; p < S.up_ptr[j + 1] && closed; p++)
            for (long long r = S.og_ptr[p]; r < S.og_ptr[p + 1]; r++)
                if (S.og_a[r] >= S.up_ptr[j] || S.og_b[r] >= S.up_ptr[j]) { closed = false; break; }
    info[0] = S.n;
    info[1] = S.nup;
    info[2] = S.pairs();
    info[3] = (long long)S.flev_ptr.size() - 1;
    info[4] = (long long)S.blev_ptr.size() - 1;
    info[5] = y.nnz;
    info[6] = jblocks;
    info[7] = closed ? 1 : 0;
    return GBPF_OK;
}
