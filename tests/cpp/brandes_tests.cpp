// The reference's Brandes unit tests (libfastbc/test/brandes/*.cpp), restated against the
// GPU engines of include/fastbc_gpu/engine.hpp.  The graph types here are small test
// doubles with the reference's IGraph/ISubGraph surface (vertices, forwardStar, borders,
// referenceGraph); the fixture is the reference's DWGtext.txt.
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
            // "Dijkstra cluster evaluation test" (DijkstraClusterEvaluator.cpp:15-109)
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
