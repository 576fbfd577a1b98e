// Test infrastructure only: a driver that runs the UNMODIFIED reference fast-bc
// headers (libfastbc/include, compiled in place from the read-only reference tree)
// on an edge-list file and dumps their results at full precision, so that the
// oracle restatement and the golden fixtures can be pinned to the reference itself.
//
// Modes (all single-threaded unless OMP_NUM_THREADS says otherwise):
//   exact     <edges> <out>                      ExactBrandesBC::computeBC        (ExactBrandesBC.h:45-95)
//   ss        <edges> <src> <out>                DijkstraSSBrandesBC::singleSourceBrandes (DijkstraSSBrandesBC.h:45-81)
//   cluster   <edges> <verts> <out_prefix>       SubGraph + DijkstraClusterEvaluator (DijkstraClusterEvaluator.h:50-180)
//   clustered <edges> <seeds> <prec> <kfrac> <out_prefix>
//             replays ClusteredBrandeBC::computeBC step by step (ClusteredBrandesBC.h:63-169),
//             dumping the partition, borders, pivots and cardinalities, the intra-cluster
//             BC and the final BC, and also runs computeBC itself to cross-check the replay.
//   partition <edges> <seeds> <prec> <out>          LouvainGraphPartition alone: the communities
//   select    <edges> <kfrac> <cluster.bin>...      KMeansPivotSelector on clusters evaluated elsewhere
//   classes   <edges> <clusters> <out_prefix>       cluster evaluation + VertexInfoPivotSelector per
//                                                   cluster (clusters file: one line per cluster,
//                                                   "count v1 v2 ..."): exact classes' pivots/sizes
//   graph     <edges> <out>                         DirectedWeightedGraph(std::istream&) alone: "n m",
//                                                   then "src dst weight" per edge in forward-star
//                                                   order, or "error <what()>" when it throws
//   pins                                            the reference unit-test scenarios on DWGtext
#define FASTBC_BRANDES_ENABLE_PIVOT_BORDER
#define FASTBC_BRANDES_CLUSTERED_IGNORE_UNCONNECTED
#include <limits>
#include <stdexcept>
#include <set>
#include <map>
#include <sstream>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include <DirectedWeightedGraph.h>
#include <SubGraph.h>
#include <brandes/ClusteredBrandesBC.h>
#include <brandes/DijkstraClusterEvaluator.h>
#include <brandes/DijkstraSSBrandesBC.h>
#include <brandes/ExactBrandesBC.h>
#include <brandes/KMeansPivotSelector.h>
#include <brandes/VertexInfoPivotSelector.h>
#include <kmeans/PlusPlusKMeans.h>
#include <louvain/LouvainGraphPartition.h>

using V = int;
using W = double;
using Graph = fastbc::DirectedWeightedGraph<V, W>;

static std::shared_ptr<Graph> load(const char* path) {
    std::ifstream f(path);
    if (!f.is_open()) throw std::runtime_error(std::string("cannot open ") + path);
    return std::make_shared<Graph>(f);
}

static void dump_vec(const char* path, const std::vector<W>& v) {
    FILE* f = std::fopen(path, "w");
    for (double x : v) std::fprintf(f, "%.17g\n", x);
    std::fclose(f);
}

static std::vector<V> read_ints(const char* path) {
    std::ifstream f(path);
    std::vector<V> out;
    V x;
    while (f >> x) out.push_back(x);
    return out;
}

// one cluster per line: "count v1 v2 ..."
static std::vector<std::vector<V>> read_clusters(const char* path) {
    std::ifstream f(path);
    std::vector<std::vector<V>> out;
    size_t k;
    while (f >> k) {
        std::vector<V> c(k);
        for (auto& v : c) f >> v;
        out.push_back(std::move(c));
    }
    return out;
}

int main(int argc, char** argv) {
    if (argc < 2) { std::fprintf(stderr, "usage: see header\n"); return 2; }
    std::string mode = argv[1];
    if (mode == "graph" && argc == 4) {
        std::FILE* o = std::fopen(argv[3], "w");
        try {
            auto g = load(argv[2]);
            std::fprintf(o, "%zu %d\n", g->vertices().size(), (int)g->edges());
            for (V v : g->vertices())
                for (const auto& e : g->forwardStar(v)) std::fprintf(o, "%d %d %.17g\n", v, e.first, e.second);
        } catch (const std::exception& e) {
            std::fprintf(o, "error %s\n", e.what());
        }
        std::fclose(o);
        return 0;
    }
    if (mode == "exact" && argc == 4) {
        auto g = load(argv[2]);
        fastbc::brandes::ExactBrandesBC<V, W> bc;
        dump_vec(argv[3], bc.computeBC(g));
        return 0;
    }
    if (mode == "ss" && argc == 5) {
        auto g = load(argv[2]);
        fastbc::brandes::DijkstraSSBrandesBC<V, W> ss;
        dump_vec(argv[4], ss.singleSourceBrandes(std::atoi(argv[3]), g));
        return 0;
    }
    if (mode == "cluster" && argc == 5) {
        auto g = load(argv[2]);
        std::vector<V> verts = read_ints(argv[3]);
        auto sg = std::make_shared<fastbc::SubGraph<V, W>>(verts, g);
        std::vector<W> bc(g->vertices().size(), 0.0);
        std::vector<std::shared_ptr<fastbc::brandes::VertexInfo<V, W>>> vi(g->vertices().size(), nullptr);
        fastbc::brandes::DijkstraClusterEvaluator<V, W> ce;
        ce.evaluateCluster(bc, vi, sg);
        std::string pre = argv[4];
        dump_vec((pre + ".bc").c_str(), bc);
        FILE* f = std::fopen((pre + ".vi").c_str(), "w");
        std::fprintf(f, "%zu\n", sg->borders().size());
        for (V b : sg->borders()) std::fprintf(f, "%d ", b);
        std::fprintf(f, "\n");
        for (V v : verts) {
            auto& x = vi[v];
            for (int i = 0; i < x->borders(); ++i)
                std::fprintf(f, "%.17g %d ", x->getBorderSPLength(i), x->getBorderSPCount(i));
            std::fprintf(f, "\n");
        }
        std::fclose(f);
        return 0;
    }
    if (mode == "partition" && argc == 6) {
        // LouvainGraphPartition::partitionGraph alone (ClusteredBrandesBC.h:80-81): one line per
        // community, its vertices in the reference's order.
        auto g = load(argv[2]);
        std::set<std::mt19937::result_type> seeds;
        {
            std::stringstream ss(argv[3]);
            std::mt19937::result_type s;
            while (ss >> s) { seeds.insert(s); if (ss.peek() == ',') ss.ignore(); }
        }
        auto gp = std::make_shared<fastbc::louvain::LouvainGraphPartition<V, W>>(seeds, std::atof(argv[4]));
        auto comms = gp->partitionGraph(std::static_pointer_cast<const fastbc::IDegreeGraph<V, W>>(g));
        FILE* f = std::fopen(argv[5], "w");
        std::fprintf(f, "%zu\n", comms.size());
        for (const auto& c : comms) {
            std::fprintf(f, "%zu", c.size());
            for (V v : c) std::fprintf(f, " %d", v);
            std::fprintf(f, "\n");
        }
        std::fclose(f);
        return 0;
    }
    if (mode == "classes" && argc == 5) {
        // VertexInfoPivotSelector::selectPivots (VertexInfoPivotSelector.h:30-123) on every
        // cluster of a given partition, after DijkstraClusterEvaluator::evaluateCluster: the exact
        // topological classes' pivots and cardinalities, per cluster, plus the intra-cluster BC.
        auto g = load(argv[2]);
        auto clusters = read_clusters(argv[3]);
        std::string pre = argv[4];
        const size_t n = g->vertices().size();
        std::vector<W> bc(n, 0.0);
        std::vector<std::shared_ptr<fastbc::brandes::VertexInfo<V, W>>> vi(n, nullptr);
        fastbc::brandes::DijkstraClusterEvaluator<V, W> ce;
        fastbc::brandes::VertexInfoPivotSelector<V, W> ps;
        std::vector<std::shared_ptr<fastbc::SubGraph<V, W>>> sgs;
        for (auto& c : clusters) {
            sgs.push_back(std::make_shared<fastbc::SubGraph<V, W>>(c, g));
            if (!sgs.back()->borders().empty()) ce.evaluateCluster(bc, vi, sgs.back());
        }
        dump_vec((pre + ".intra").c_str(), bc);
        FILE* f = std::fopen((pre + ".classes").c_str(), "w");
        for (auto& sg : sgs) {
            if (sg->borders().empty()) { std::fprintf(f, "0\n0\n"); continue; }
            auto piv = ps.selectPivots(bc, vi, sg->vertices(), sg->borders());
            std::fprintf(f, "%zu", piv.first.size());
            for (V v : piv.first) std::fprintf(f, " %d", v);
            std::fprintf(f, "\n%zu", piv.second.size());
            for (V k : piv.second) std::fprintf(f, " %d", k);
            std::fprintf(f, "\n");
        }
        std::fclose(f);
        return 0;
    }
    if (mode == "select" && argc >= 5) {
        // KMeansPivotSelector (VertexInfoPivotSelector + PlusPlusKMeans, KMeansPivotSelector.h:79-132)
        // on clusters whose intra-cluster BC and border vectors were computed elsewhere (the oracle,
        // bit-identical to DijkstraClusterEvaluator): one binary file per cluster, "int64 nc,
        // int64 nb, int32 vertices[nc], double bc[nc], double len[nc*nb], double sigma[nc*nb]"; the
        // borders are the reference SubGraph's own.  Prints per cluster "file count pivots..." and
        // "count cards..." lines.
        auto g = load(argv[2]);
        const double kfrac = std::atof(argv[3]);
        const size_t n = g->vertices().size();
        for (int a = 4; a < argc; ++a) {
            FILE* f = std::fopen(argv[a], "rb");
            if (!f) throw std::runtime_error(std::string("cannot open ") + argv[a]);
            int64_t nc = 0, nb = 0;
            if (std::fread(&nc, 8, 1, f) != 1 || std::fread(&nb, 8, 1, f) != 1) throw std::runtime_error("short file");
            std::vector<V> verts(nc);
            std::vector<double> cbc(nc), len(nc * nb), sig(nc * nb);
            if (std::fread(verts.data(), 4, nc, f) != (size_t)nc || std::fread(cbc.data(), 8, nc, f) != (size_t)nc ||
                std::fread(len.data(), 8, nc * nb, f) != (size_t)(nc * nb) ||
                std::fread(sig.data(), 8, nc * nb, f) != (size_t)(nc * nb))
                throw std::runtime_error("short file");
            std::fclose(f);
            auto sg = std::make_shared<fastbc::SubGraph<V, W>>(verts, g);
            if ((int64_t)sg->borders().size() != nb) throw std::runtime_error("border count differs");
            std::vector<W> bc(n, 0.0);
            std::vector<std::shared_ptr<fastbc::brandes::VertexInfo<V, W>>> vi(n, nullptr);
            for (int64_t i = 0; i < nc; ++i) {
                bc[verts[i]] = cbc[i];
                vi[verts[i]] = std::make_shared<fastbc::brandes::VertexInfo<V, W>>((int)nb);
                for (int64_t j = 0; j < nb; ++j) {
                    // the same W -> V conversions as DijkstraClusterEvaluator.h:173-174
                    vi[verts[i]]->setBorderSPLength((int)j, len[i * nb + j]);
                    vi[verts[i]]->setBorderSPCount((int)j, sig[i * nb + j]);
                }
            }
            fastbc::brandes::KMeansPivotSelector<V, W> ps(
                std::shared_ptr<fastbc::brandes::IPivotSelector<V, W>>(new fastbc::brandes::VertexInfoPivotSelector<V, W>()),
                std::shared_ptr<fastbc::kmeans::IKMeans<V, W>>(new fastbc::kmeans::PlusPlusKMeans<V, W>()), kfrac);
            auto piv = ps.selectPivots(bc, vi, sg->vertices(), sg->borders());
            std::printf("%s %zu", argv[a], piv.first.size());
            for (V v : piv.first) std::printf(" %d", v);
            std::printf("\n%zu", piv.second.size());
            for (V k : piv.second) std::printf(" %d", k);
            std::printf("\n");
            std::fflush(stdout);
        }
        return 0;
    }
    if (mode == "clustered" && argc == 7) {
        auto g = load(argv[2]);
        std::set<std::mt19937::result_type> seeds;
        {
            std::stringstream ss(argv[3]);
            std::mt19937::result_type s;
            while (ss >> s) { seeds.insert(s); if (ss.peek() == ',') ss.ignore(); }
        }
        double prec = std::atof(argv[4]);
        double kfrac = std::atof(argv[5]);
        std::string pre = argv[6];
        using namespace fastbc;
        using namespace fastbc::brandes;
        auto gp = std::make_shared<louvain::LouvainGraphPartition<V, W>>(seeds, prec);
        auto ce = std::make_shared<DijkstraClusterEvaluator<V, W>>();
        std::shared_ptr<IPivotSelector<V, W>> ps;
        if (kfrac > 0)
            ps = std::make_shared<KMeansPivotSelector<V, W>>(
                std::shared_ptr<IPivotSelector<V, W>>(new VertexInfoPivotSelector<V, W>()),
                std::shared_ptr<kmeans::IKMeans<V, W>>(new kmeans::PlusPlusKMeans<V, W>()), kfrac);
        else
            ps = std::make_shared<VertexInfoPivotSelector<V, W>>();
        auto ssb = std::make_shared<DijkstraSSBrandesBC<V, W>>();

        // Step-by-step replay of ClusteredBrandesBC.h:63-166 (single thread) capturing intermediates.
        const size_t n = g->vertices().size();
        std::vector<W> globalBC(n, 0.0);
        std::vector<std::shared_ptr<VertexInfo<V, W>>> vi(n, nullptr);
        auto comms = gp->partitionGraph(std::static_pointer_cast<const IDegreeGraph<V, W>>(g));
        std::vector<std::shared_ptr<ISubGraph<V, W>>> cl(comms.size());
        std::vector<std::pair<std::vector<V>, std::vector<V>>> piv(comms.size());
        for (size_t i = 0; i < cl.size(); ++i) {
            cl[i] = std::make_shared<SubGraph<V, W>>(comms[i], g);
            if (!cl[i]->borders().empty()) {
                ce->evaluateCluster(globalBC, vi, cl[i]);
                piv[i] = ps->selectPivots(globalBC, vi, cl[i]->vertices(), cl[i]->borders());
            }
        }
        std::vector<W> intra(globalBC);
        dump_vec((pre + ".intra").c_str(), intra);
        for (size_t c = 0; c < cl.size(); ++c) {
            for (size_t p = 0; p < piv[c].first.size(); ++p) {
                auto dep = ssb->singleSourceBrandes(piv[c].first[p], g);
                for (size_t v = 0; v < n; ++v) globalBC[v] += dep[v] * (W)(piv[c].second[p]);
                for (V v : cl[c]->vertices()) globalBC[v] -= intra[v] * (W)(piv[c].second[p]);
            }
        }
        dump_vec((pre + ".bc").c_str(), globalBC);
        FILE* f = std::fopen((pre + ".clusters").c_str(), "w");
        std::fprintf(f, "%zu\n", cl.size());
        for (size_t c = 0; c < cl.size(); ++c) {
            std::fprintf(f, "%zu", cl[c]->vertices().size());
            for (V v : cl[c]->vertices()) std::fprintf(f, " %d", v);
            std::fprintf(f, "\n%zu", cl[c]->borders().size());
            for (V v : cl[c]->borders()) std::fprintf(f, " %d", v);
            std::fprintf(f, "\n%zu", piv[c].first.size());
            for (size_t p = 0; p < piv[c].first.size(); ++p) std::fprintf(f, " %d", piv[c].first[p]);
            std::fprintf(f, "\n%zu", piv[c].second.size());
            for (size_t p = 0; p < piv[c].second.size(); ++p) std::fprintf(f, " %d", piv[c].second[p]);
            std::fprintf(f, "\n");
        }
        std::fclose(f);
        // The reference's own entry point on the same inputs: must equal the replay.
        ClusteredBrandeBC<V, W> full(
            std::make_shared<louvain::LouvainGraphPartition<V, W>>(seeds, prec), ce,
            ssb,
            kfrac > 0 ? std::shared_ptr<IPivotSelector<V, W>>(std::make_shared<KMeansPivotSelector<V, W>>(
                            std::shared_ptr<IPivotSelector<V, W>>(new VertexInfoPivotSelector<V, W>()),
                            std::shared_ptr<kmeans::IKMeans<V, W>>(new kmeans::PlusPlusKMeans<V, W>()), kfrac))
                      : std::shared_ptr<IPivotSelector<V, W>>(std::make_shared<VertexInfoPivotSelector<V, W>>()));
        dump_vec((pre + ".bc_ref").c_str(), full.computeBC(g));
        return 0;
    }
    if (mode == "pins" && argc == 3) {
        // The scenarios of libfastbc/test/brandes/{ExactBrandesBC,DijkstraClusterEvaluator}.cpp,
        // run with W=float as the reference tests do, printed for the fixture generator.
        std::ifstream f1(argv[2]);
        auto fg = std::make_shared<fastbc::DirectedWeightedGraph<int, float>>(f1);
        auto sg = std::make_shared<fastbc::SubGraph<int, float>>(std::vector<int>({0, 1, 2, 3, 4}), fg);
        fastbc::brandes::ExactBrandesBC<int, float> ex;
        auto bc = ex.computeBC(sg);
        std::printf("exact_subgraph");
        for (float x : bc) std::printf(" %.9g", x);
        std::printf("\n");
        std::vector<float> gbc(fg->vertices().size(), 0.0f);
        std::vector<std::shared_ptr<fastbc::brandes::VertexInfo<int, float>>> vi(fg->vertices().size(), nullptr);
        fastbc::brandes::DijkstraClusterEvaluator<int, float> ce;
        ce.evaluateCluster(gbc, vi, sg);
        std::printf("cluster_bc");
        for (float x : gbc) std::printf(" %.9g", x);
        std::printf("\n");
        for (int v = 0; v < 5; ++v) {
            std::printf("vi %d", v);
            for (int i = 0; i < vi[v]->borders(); ++i)
                std::printf(" %.9g %d", vi[v]->getBorderSPLength(i), vi[v]->getBorderSPCount(i));
            std::printf("\n");
        }
        return 0;
    }
    std::fprintf(stderr, "bad arguments\n");
    return 2;
}
