// The clustered orchestration that GpuClusteredBrandesBC runs (fbcgpu::clustered_bc of
// include/fastbc_gpu/engine.hpp), executed with stand-ins for the host parts the reference
// supplies: the partition and the pivot selection return the reference's own choices read from
// a file (its Louvain communities and k-means pivots of the 256x256 grid), the cluster type
// computes SubGraph's border set (SubGraph.h:70-135), and the vertex-info type has the
// reference's setter signatures setBorderSPLength(int, W) / setBorderSPCount(int, V)
// (VertexInfo.h:207-244).  Writes the BC to a file (%.17g) for the test to compare with the
// reference's own ClusteredBrandeBC::computeBC result.
//
//   clustered_run <edges.txt> <clusters.txt> <out.txt>
// clusters.txt: per cluster three lines, "k v1..vk", "p pivot1..pivotp", "p card1..cardp".
#include <fastbc_gpu/engine.hpp>

#include <cstdio>
#include <fstream>
#include <map>
#include <memory>
#include <set>
#include <vector>

using V = int;
using W = double;

// DirectedWeightedGraph stand-in: the parse rules of DirectedWeightedGraph.h:67-96.
struct MapGraph {
    std::vector<V> verts;
    std::vector<std::map<V, W>> fs;
    explicit MapGraph(std::istream& in) {
        V s, d;
        W w;
        while (in >> s >> d >> w) {
            if ((V)fs.size() <= s) fs.resize(s + 1);
            fs[s][d] += w;
        }
        for (V v = 0; v < (V)fs.size(); ++v) verts.push_back(v);
    }
    const std::vector<V>& vertices() const { return verts; }
    const std::map<V, W>& forwardStar(V v) const { return fs[v]; }
    int edges() const {
        int m = 0;
        for (const auto& s : fs) m += (int)s.size();
        return m;
    }
};

// The part of SubGraph the orchestration reads: its vertices and its borders, the vertices with
// an edge crossing the cluster in either direction.
struct Cluster {
    std::vector<V> verts;
    std::set<V> bord;
    Cluster(const std::vector<V>& v, const MapGraph& g, const std::vector<int>& member_of, int id) : verts(v) {
        for (V x = 0; x < (V)g.fs.size(); ++x)
            for (const auto& e : g.fs[x]) {
                const bool a = member_of[x] == id, b = member_of[e.first] == id;
                if (a != b) bord.insert(a ? x : e.first);
            }
    }
    const std::vector<V>& vertices() const { return verts; }
    const std::set<V>& borders() const { return bord; }
};

// VertexInfo stand-in with the reference's setters.
struct Info {
    std::vector<W> len;
    std::vector<V> cnt;
    explicit Info(int nb) : len((size_t)nb, 0), cnt((size_t)nb, 0) {}
    void setBorderSPLength(int i, W l) { len.at((size_t)i) = l; }
    void setBorderSPCount(int i, V c) { cnt.at((size_t)i) = c; }
};

int main(int argc, char** argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: clustered_run <edges> <clusters> <out>\n");
        return 2;
    }
    std::ifstream gin(argv[1]);
    MapGraph g(gin);
    std::ifstream cin_(argv[2]);
    std::vector<std::vector<V>> comms, pivots, cards;
    size_t k;
    while (cin_ >> k) {
        comms.emplace_back(k);
        for (auto& v : comms.back()) cin_ >> v;
        cin_ >> k;
        pivots.emplace_back(k);
        for (auto& v : pivots.back()) cin_ >> v;
        cin_ >> k;
        cards.emplace_back(k);
        for (auto& v : cards.back()) cin_ >> v;
    }
    std::vector<int> member_of(g.fs.size(), -1);
    for (size_t c = 0; c < comms.size(); ++c)
        for (V v : comms[c]) member_of[(size_t)v] = (int)c;
    int made = 0, selected = 0, infos_missing = 0;
    fbcgpu::Options o;
    o.precision = FBC_PREC_FP64;
    const std::vector<W> bc = fbcgpu::clustered_bc<V, W>(
        g, [&](const MapGraph&) { return comms; },
        [&](const std::vector<V>& c) { return std::make_shared<Cluster>(c, g, member_of, made++); },
        [](int nb) { return std::make_shared<Info>(nb); },
        [&](const std::vector<W>&, const std::vector<std::shared_ptr<Info>>& vi, const std::vector<V>& vertices,
            const std::set<V>& borders) {
            for (V v : vertices)
                if (!vi[(size_t)v] || vi[(size_t)v]->len.size() != borders.size()) ++infos_missing;
            const int c = member_of[(size_t)vertices[0]];
            ++selected;
            return std::make_pair(pivots[(size_t)c], cards[(size_t)c]);
        },
        o, true);
    FILE* f = std::fopen(argv[3], "w");
    for (W x : bc) std::fprintf(f, "%.17g\n", x);
    std::fclose(f);
    std::printf("clusters %zu selected %d infos_missing %d\n", comms.size(), selected, infos_missing);
    return infos_missing == 0 ? 0 : 1;
}
