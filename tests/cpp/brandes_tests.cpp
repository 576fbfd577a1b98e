// The reference's Brandes unit tests (libfastbc/test/brandes/*.cpp), restated against the
// GPU engines of include/fastbc_gpu/engine.hpp.  The graph types here are small test
// doubles with the reference's IGraph/ISubGraph surface (vertices, forwardStar, borders,
// referenceGraph); the fixture is the reference's DWGtext.txt.
#include <algorithm>
#include <fastbc_gpu/engine.hpp>

#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <memory>
#include <set>
#include <vector>

static int g_fail = 0;
#define REQUIRE(c)                                                         \
    do {                                                                   \
        if (!(c)) {                                                        \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);     \
            ++g_fail;                                                      \
        }                                                                  \
    } while (0)

// DirectedWeightedGraph stand-in: parse rules of DirectedWeightedGraph.h:67-96.
struct MapGraph {
    std::vector<int> verts;
    std::vector<std::map<int, double>> fs;
    explicit MapGraph(std::istream& in) {
        int s, d;
        double w;
        while (in >> s >> d >> w) {
            if ((int)fs.size() <= s) fs.resize(s + 1);
            fs[s][d] += w;
        }
        for (int v = 0; v < (int)fs.size(); ++v) verts.push_back(v);
    }
    const std::vector<int>& vertices() const { return verts; }
    const std::map<int, double>& forwardStar(int v) const { return fs[v]; }
    int edges() const {
        int m = 0;
        for (const auto& s : fs) m += (int)s.size();
        return m;
    }
};

// SubGraph stand-in: induced subgraph with border set (SubGraph.h:59-148).
struct MapSubGraph {
    std::vector<int> verts;
    std::set<int> bord;
    std::vector<std::map<int, double>> fs;
    std::shared_ptr<const MapGraph> ref;
    MapSubGraph(std::vector<int> v, std::shared_ptr<const MapGraph> g) : verts(v), ref(g) {
        std::set<int> in(v.begin(), v.end());
        fs.resize(g->fs.size());
        for (int x = 0; x < (int)g->fs.size(); ++x)
            for (auto& e : g->fs[x]) {
                bool a = in.count(x), b = in.count(e.first);
                if (a && b) fs[x][e.first] = e.second;
                if (a != b) bord.insert(a ? x : e.first);
            }
    }
    const std::vector<int>& vertices() const { return verts; }
    const std::map<int, double>& forwardStar(int v) const { return fs[v]; }
    int edges() const {
        int m = 0;
        for (int v : verts) m += (int)fs[v].size();
        return m;
    }
    const std::set<int>& borders() const { return bord; }
    std::shared_ptr<const MapGraph> referenceGraph() const { return ref; }
};

// VertexInfo stand-in (VertexInfo.h): border path lengths (W) and counts (V); normalize subtracts
// the least length (VertexInfo.h:259-278).
struct MiniVI {
    std::vector<double> len;
    std::vector<int> cnt;
    MiniVI(std::vector<double> l, std::vector<int> c) : len(std::move(l)), cnt(std::move(c)) {}
    int borders() const { return (int)len.size(); }
    double getBorderSPLength(int j) const { return len[j]; }
    int getBorderSPCount(int j) const { return cnt[j]; }
    void normalize() {
        if (len.empty()) return;
        const double m = *std::min_element(len.begin(), len.end());
        for (double& x : len) x -= m;
    }
};

int main(int argc, char** argv) {
    std::ifstream f(argc > 1 ? argv[1] : "DWGtext.txt");
    auto full = std::make_shared<MapGraph>(f);
    REQUIRE(full->vertices().size() == 9);
    MapSubGraph sub({0, 1, 2, 3, 4}, full);
    for (int prec : {FBC_PREC_FP64, FBC_PREC_FP32C})
        for (int sched : {FBC_SCHED_PLAIN, FBC_SCHED_BATCHED}) {
            fbcgpu::Options o;
            o.precision = prec;
            o.sched = sched;
            // "Exact Brandes' BC computation test" (ExactBrandesBC.cpp:11-35), on the subgraph
            auto bc = fbcgpu::exact_bc<float>(sub, o);
            REQUIRE(bc.size() == sub.vertices().size());  // sized as ExactBrandesBC.h:49 sizes it
            REQUIRE(bc[0] == 2.0f);
            REQUIRE(bc[1] == 2.0f);
            REQUIRE(bc[2] == 0.5f);
            REQUIRE(bc[3] == 1.0f);
            REQUIRE(bc[4] == 0.0f);
            // "Dijkstra cluster evaluation test" (DijkstraClusterEvaluator.cpp:15-74)
            auto d = fbcgpu::DeviceGraph::from_graph(*full);
            std::vector<std::vector<int32_t>> cv{{0, 1, 2, 3, 4}}, bv{{3, 4}};
            std::vector<double> len;
            std::vector<uint64_t> cnt;
            auto cbc = fbcgpu::cluster_eval_batch(*d, cv, bv, o, &len, &cnt, nullptr);
            REQUIRE(cbc[0] == 2.0 && cbc[1] == 2.0 && cbc[2] == 0.5 && cbc[3] == 1.0 && cbc[4] == 0.0);
            for (int i = 5; i < 9; ++i) REQUIRE(cbc[i] == 0.0);
            const double L[5][2] = {{5, 7}, {1, 4}, {8, 4}, {0, 3}, {0, 0}};
            const int K[5][2] = {{1, 2}, {1, 1}, {1, 1}, {1, 1}, {0, 1}};
            for (int v = 0; v < 5; ++v)
                for (int j = 0; j < 2; ++j) {
                    REQUIRE(len[v * 2 + j] == L[v][j]);
                    REQUIRE((int)cnt[v * 2 + j] == K[v][j]);
                }
            // "Single source Brandes BC" (DijkstraSSBrandesBC.cpp:12-28): size, plus values
            auto dep = fbcgpu::single_source<double>(*d, 0, o);
            REQUIRE(dep.size() == full->vertices().size());
            const double want[9] = {0, 3.3333333333333335, 1.3333333333333333, 2.3333333333333335,
                                    1.6666666666666667, 1.3333333333333333, 0, 0, 0};
            for (int v = 0; v < 9; ++v) REQUIRE(std::fabs(dep[v] - want[v]) <= 1e-9 * std::fabs(want[v]));
        }
    // the device graph parsed from the file stands for the host graph read from it: the same
    // CSR as the upload of the host graph's stars, used by the engines given that host object
    {
        auto dg = fbcgpu::DeviceGraph::from_file(argc > 1 ? argv[1] : "DWGtext.txt");
        auto up = fbcgpu::DeviceGraph::from_graph(*full);
        std::vector<int64_t> rp1, rp2;
        std::vector<int32_t> c1, c2;
        std::vector<double> w1, w2;
        dg->download_csr(rp1, c1, w1);
        up->download_csr(rp2, c2, w2);
        REQUIRE(rp1 == rp2 && c1 == c2 && w1 == w2);
        fbcgpu::Options o;
        auto before = fbcgpu::exact_bc<double>(*full, o);
        fbcgpu::use_device_graph(full.get(), dg);
        REQUIRE(fbcgpu::device_graph_for(*full, 0) == dg);
        auto after = fbcgpu::exact_bc<double>(*full, o);
        REQUIRE(before == after);
        bool mismatch = false;  // a preload for an object with other counts is refused
        fbcgpu::use_device_graph(&sub, dg);
        try {
            fbcgpu::exact_bc<double>(sub, o);
        } catch (const fbcgpu::Error& e) {
            mismatch = e.code == FBC_ERR_INVALID_ARG;
        }
        REQUIRE(mismatch);
        fbcgpu::use_device_graph(nullptr, nullptr);
    }
    // "Pivot selection" (VertexInfoPivotSelector.cpp:14-74) with the class grouping on the device:
    // that test's global BC and the first two border entries of its vertex infos, borders {0, 4}.
    // Normalized: v0 (0,1 | 2,1), v1 (1,0 | 2,2), v2 (0,1 | 2,1), v3 (1,0 | 2,2), v4 (4,0 | 1,1):
    // classes {0,2}, {1,3}, {4}; pivots the least-BC non-border member (2; 3 with BC 1.5 < 2),
    // and for the all-border class {4} its first member, or none.
    {
        std::vector<double> gbc{1, 2, 2, 1.5, 1, 3};
        auto make = [] {
            std::vector<std::shared_ptr<MiniVI>> vi;
            vi.push_back(std::make_shared<MiniVI>(std::vector<double>{1, 2}, std::vector<int>{2, 1}));
            vi.push_back(std::make_shared<MiniVI>(std::vector<double>{2, 1}, std::vector<int>{2, 2}));
            vi.push_back(std::make_shared<MiniVI>(std::vector<double>{2, 3}, std::vector<int>{2, 1}));
            vi.push_back(std::make_shared<MiniVI>(std::vector<double>{4, 3}, std::vector<int>{2, 2}));
            vi.push_back(std::make_shared<MiniVI>(std::vector<double>{5, 1}, std::vector<int>{1, 1}));
            vi.push_back(nullptr);
            return vi;
        };
        std::vector<int> verts{0, 1, 2, 3, 4};
        std::set<int> bord{0, 4};
        auto vi = make();
        REQUIRE(fbcgpu::use_device_classes(vi, verts, bord));
        auto p = fbcgpu::select_pivots<int, double>(gbc, vi, verts, bord, true);
        REQUIRE((p.first == std::vector<int>{2, 3, 4}) && (p.second == std::vector<int>{2, 2, 1}));
        REQUIRE(vi[3]->len[0] == 1.0 && vi[3]->len[1] == 0.0);  // normalized in place, as the reference does
        vi = make();
        p = fbcgpu::select_pivots<int, double>(gbc, vi, verts, bord, false);
        REQUIRE((p.first == std::vector<int>{2, 3}) && (p.second == std::vector<int>{2, 2}));
        // outside the pipeline's shape (the reference test's empty border set with 3-entry infos):
        // the device path does not apply
        REQUIRE(!fbcgpu::use_device_classes(vi, verts, std::set<int>{}));
    }
    // invalid input is reported as an exception carrying the library's status
    bool threw = false;
    try {
        int64_t rp[3] = {0, 1, 2};
        int32_t col[2] = {1, 0};
        double w[2] = {1.0, -2.0};
        fbc_graph h = nullptr;
        fbcgpu::check(fbc_graph_upload(2, rp, col, w, &h));
    } catch (const fbcgpu::Error& e) {
        threw = e.code == FBC_ERR_INVALID_ARG;
    }
    REQUIRE(threw);
    std::printf(g_fail ? "C++ tests: %d failures\n" : "C++ tests: all passed\n", g_fail);
    return g_fail ? 1 : 0;
}
