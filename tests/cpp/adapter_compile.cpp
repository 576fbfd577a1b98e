// Compile-and-link check of the drop-in classes against the reference's own headers
// (built only where the reference tree is present; the checks run nothing on a GPU).
// It also wires them exactly as the fbc CLI wires the CPU classes (main.cpp:214-260).
#define FASTBC_BRANDES_ENABLE_PIVOT_BORDER
#define FASTBC_BRANDES_CLUSTERED_IGNORE_UNCONNECTED
#include <DirectedWeightedGraph.h>
#include <brandes/ClusteredBrandesBC.h>
#include <brandes/DijkstraClusterEvaluator.h>
#include <brandes/DijkstraSSBrandesBC.h>
#include <brandes/ExactBrandesBC.h>
#include <brandes/KMeansPivotSelector.h>
#include <brandes/VertexInfoPivotSelector.h>
#include <kmeans/PlusPlusKMeans.h>
#include <louvain/LouvainGraphPartition.h>

#include <fastbc_gpu/fastbc_adapters.hpp>

#include <cstdio>
#include <fstream>

using V = int;
using W = double;
using namespace fastbc;
using namespace fastbc::brandes;

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    std::ifstream f(argv[1]);
    std::shared_ptr<IGraph<V, W>> graph = std::make_shared<DirectedWeightedGraph<V, W>>(f);
    fbcgpu::Options o;
    o.precision = FBC_PREC_FP64;
    std::shared_ptr<IBrandesBC<V, W>> exact = std::make_shared<GpuExactBrandesBC<V, W>>(o);
    std::set<std::mt19937::result_type> seeds{1, 2, 3, 4};
    auto gp = std::make_shared<louvain::LouvainGraphPartition<V, W>>(seeds, 0.01);
    std::shared_ptr<IPivotSelector<V, W>> ps = std::make_shared<KMeansPivotSelector<V, W>>(
        std::shared_ptr<IPivotSelector<V, W>>(new VertexInfoPivotSelector<V, W>()),
        std::shared_ptr<kmeans::IKMeans<V, W>>(new kmeans::PlusPlusKMeans<V, W>()), 0.5);
    // reference orchestration with GPU strategy objects
    std::shared_ptr<IBrandesBC<V, W>> clustered = std::make_shared<ClusteredBrandeBC<V, W>>(
        gp, std::make_shared<GpuClusterEvaluator<V, W>>(o), std::make_shared<GpuSSBrandesBC<V, W>>(o), ps);
    // batched GPU orchestration
    std::shared_ptr<IBrandesBC<V, W>> batched = std::make_shared<GpuClusteredBrandesBC<V, W>>(gp, ps, o);
    // the exact class grouping on the device inside the reference's k-means selector
    std::shared_ptr<IPivotSelector<V, W>> gps = std::make_shared<KMeansPivotSelector<V, W>>(
        std::make_shared<GpuVertexInfoPivotSelector<V, W>>(o),
        std::shared_ptr<kmeans::IKMeans<V, W>>(new kmeans::PlusPlusKMeans<V, W>()), 0.5);
    std::shared_ptr<IBrandesBC<V, W>> batched_gps = std::make_shared<GpuClusteredBrandesBC<V, W>>(gp, gps, o);
    (void)batched_gps;
    // and the k-means step on the device too
    std::shared_ptr<IPivotSelector<V, W>> gkm = std::make_shared<KMeansPivotSelector<V, W>>(
        std::make_shared<GpuVertexInfoPivotSelector<V, W>>(o),
        std::make_shared<kmeans::GpuPlusPlusKMeans<V, W>>(o), 0.5);
    (void)gkm;
    if (argc > 2) {
        std::string mode = argv[2];
        std::vector<W> bc = mode == "exact" ? exact->computeBC(graph)
                            : mode == "clustered" ? clustered->computeBC(graph)
                                                  : batched->computeBC(graph);
        for (double x : bc) std::printf("%.17g\n", x);
    }
    return 0;
}
