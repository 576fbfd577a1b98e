// The host locality order (fast-bc_gb300/csrc/host_order.hpp): the thread-pool bisection gives the
// same permutation as the plain sequential recursion restated here, for graphs with several
// components, long paths, empty and tiny graphs; and on a road-like grid it keeps more edges
// within short id distances than the input order does.
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <random>
#include <vector>

#include "host_order.hpp"

namespace {

// the sequential recursion: a range laid out in BFS order (each not yet reached vertex of the
// range in turn, edges followed inside the range), then halved; ranges of at most `leaf` sorted
std::vector<int32_t> order_seq(int32_t n, const std::vector<int64_t>& rp, const std::vector<int32_t>& col, int leaf) {
    std::vector<int32_t> ord(n), q;
    std::iota(ord.begin(), ord.end(), 0);
    std::vector<int64_t> owner(n, -1);
    std::vector<char> seen(n, 0);
    int64_t tag = 0;
    std::vector<std::pair<int64_t, int64_t>> stk{{0, n}};
    while (!stk.empty()) {
        auto [lo, hi] = stk.back();
        stk.pop_back();
        if (hi - lo <= leaf) {
            std::sort(ord.begin() + lo, ord.begin() + hi);
            continue;
        }
        ++tag;
        for (int64_t i = lo; i < hi; ++i) owner[ord[i]] = tag;
        q.clear();
        for (int64_t i = lo; i < hi; ++i) {
            if (seen[ord[i]]) continue;
            size_t h = q.size();
            q.push_back(ord[i]);
            seen[ord[i]] = 1;
            while (h < q.size()) {
                const int32_t v = q[h++];
                for (int64_t e = rp[v]; e < rp[v + 1]; ++e)
                    if (owner[col[e]] == tag && !seen[col[e]]) {
                        seen[col[e]] = 1;
                        q.push_back(col[e]);
                    }
            }
        }
        for (int64_t i = lo; i < hi; ++i) {
            ord[i] = q[i - lo];
            seen[q[i - lo]] = 0;
        }
        const int64_t mid = lo + (hi - lo) / 2;
        stk.emplace_back(mid, hi);
        stk.emplace_back(lo, mid);
    }
    std::vector<int32_t> nw(n);
    for (int32_t i = 0; i < n; ++i) nw[ord[i]] = i;
    return nw;
}

struct G {
    int32_t n = 0;
    std::vector<int64_t> rp{0};
    std::vector<int32_t> col;
};

G from_pairs(int32_t n, std::vector<std::pair<int32_t, int32_t>> e) {
    std::sort(e.begin(), e.end());
    e.erase(std::unique(e.begin(), e.end()), e.end());
    G g;
    g.n = n;
    g.rp.assign(n + 1, 0);
    for (auto& p : e) ++g.rp[p.first + 1];
    for (int32_t v = 0; v < n; ++v) g.rp[v + 1] += g.rp[v];
    for (auto& p : e) g.col.push_back(p.second);
    return g;
}

G grid(int r, int c, double drop, unsigned seed) {
    std::mt19937 rng(seed);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    std::vector<std::pair<int32_t, int32_t>> e;
    for (int i = 0; i < r; ++i)
        for (int j = 0; j < c; ++j) {
            const int32_t v = i * c + j;
            if (j + 1 < c && u(rng) >= drop) { e.emplace_back(v, v + 1); e.emplace_back(v + 1, v); }
            if (i + 1 < r && u(rng) >= drop) { e.emplace_back(v, v + c); e.emplace_back(v + c, v); }
        }
    return from_pairs(r * c, e);
}

int fails = 0;
void check(bool ok, const char* what) {
    if (!ok) {
        std::printf("FAILED: %s\n", what);
        ++fails;
    }
}

double near_fraction(const G& g, const std::vector<int32_t>& nw, int32_t span) {
    int64_t near = 0, m = 0;
    for (int32_t v = 0; v < g.n; ++v)
        for (int64_t e = g.rp[v]; e < g.rp[v + 1]; ++e, ++m) near += std::abs(nw[v] - nw[g.col[e]]) < span;
    return m ? (double)near / (double)m : 1.0;
}

}  // namespace

int main() {
    std::vector<std::pair<const char*, G>> cases;
    cases.emplace_back("empty", G{});
    cases.emplace_back("one vertex", from_pairs(1, {}));
    cases.emplace_back("isolated vertices", from_pairs(300000, {}));
    {
        std::vector<std::pair<int32_t, int32_t>> e;
        for (int32_t v = 0; v + 1 < 200000; ++v) { e.emplace_back(v, v + 1); e.emplace_back(v + 1, v); }
        cases.emplace_back("path", from_pairs(200000, e));
    }
    cases.emplace_back("grid 400x400, 5% dropped", grid(400, 400, 0.05, 1));
    cases.emplace_back("grid 300x500, 40% dropped (many components)", grid(300, 500, 0.40, 2));
    {
        std::mt19937 rng(3);
        std::uniform_int_distribution<int32_t> pick(0, 149999);
        std::vector<std::pair<int32_t, int32_t>> e;
        for (int k = 0; k < 300000; ++k) e.emplace_back(pick(rng), pick(rng));  // directed, random
        cases.emplace_back("random directed", from_pairs(150000, e));
    }
    for (auto& [name, g] : cases) {
        const auto a = fbc_host::bisection_order(g.n, g.rp, g.col, 16);
        const auto b = order_seq(g.n, g.rp, g.col, 16);
        std::vector<char> hit(g.n, 0);
        bool perm = (int32_t)a.size() == g.n;
        for (int32_t x : a) perm = perm && x >= 0 && x < g.n && !hit[x] && (hit[x] = 1);
        check(perm, name);
        check(a == b, name);
        check(a == fbc_host::bisection_order(g.n, g.rp, g.col, 16), name);  // independent of timing
    }
    {
        const G g = grid(512, 512, 0.05, 4);
        std::vector<int32_t> id(g.n);
        std::iota(id.begin(), id.end(), 0);
        const auto nw = fbc_host::bisection_order(g.n, g.rp, g.col, 16);
        const double f0 = near_fraction(g, id, 256), f1 = near_fraction(g, nw, 256);
        std::printf("edges within 256 ids: input order %.3f, locality order %.3f\n", f0, f1);
        check(f1 > f0 + 0.2, "locality");
    }
    // the parallel loop covers every index once
    std::vector<std::atomic<int>> cnt(1000003);
    fbc_host::host_parallel((int64_t)cnt.size(), [&](int64_t lo, int64_t hi) {
        for (int64_t i = lo; i < hi; ++i) cnt[i].fetch_add(1);
    });
    bool once = true;
    for (auto& c : cnt) once = once && c.load() == 1;
    check(once, "host_parallel");
    if (fails == 0) std::printf("all passed\n");
    return fails ? 1 : 0;
}
