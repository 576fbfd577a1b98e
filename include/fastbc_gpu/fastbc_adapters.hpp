// Drop-in GPU implementations of fast-bc's hot-path interfaces.
//
// Include this header AFTER the reference's own headers (it derives from their classes):
//   #include <brandes/ClusteredBrandesBC.h>   // and the other fast-bc headers fbc uses
//   #include <fastbc_gpu/fastbc_adapters.hpp>
// and link libfbcgpu.so.  Classes (namespace fastbc::brandes, same V/W templates):
//   GpuExactBrandesBC       : IBrandesBC         replaces ExactBrandesBC (ExactBrandesBC.h:45-95)
//   GpuSSBrandesBC          : ISSBrandesBC       replaces DijkstraSSBrandesBC (DijkstraSSBrandesBC.h:45-81)
//   GpuClusterEvaluator     : IClusterEvaluator  replaces DijkstraClusterEvaluator
//                                                (DijkstraClusterEvaluator.h:50-180)
//   GpuVertexInfoPivotSelector : IPivotSelector  replaces VertexInfoPivotSelector
//                                                (VertexInfoPivotSelector.h:30-123): the exact
//                                                topological classes grouped on the device (the
//                                                reference's own selector for inputs outside the
//                                                clustered pipeline's shape); usable as the
//                                                exact selector inside KMeansPivotSelector
//   GpuPlusPlusKMeans       : kmeans::IKMeans    replaces PlusPlusKMeans (PlusPlusKMeans.h:76-147) inside
//                                                KMeansPivotSelector: the same centroids and weights
//   GpuClusteredBrandesBC   : IBrandesBC         ClusteredBrandeBC (ClusteredBrandesBC.h:63-169)
//                             with one GPU call for all clusters and one for all pivots; the
//                             partition and pivot selection are the caller's reference objects.
// Contracts kept: computeBC returns a vector of size vertices().size(); singleSourceBrandes
// returns the dependency with dep[source] = 0; evaluateCluster adds into clusterBC and
// allocates globalVI[v] only for the cluster's vertices, unreached border length 0 and the
// count stored through VertexInfo::setBorderSPCount(int, V) from the W-typed count, as the
// reference does.  All of them may be called from OpenMP worker threads.
#pragma once

#include <memory>
#include <utility>
#include <vector>

#include "engine.hpp"

namespace fastbc {
namespace brandes {

template <typename V, typename W>
class GpuExactBrandesBC : public IBrandesBC<V, W> {
  public:
    explicit GpuExactBrandesBC(fbcgpu::Options o = {}) : _o(o) {}
    std::vector<W> computeBC(const std::shared_ptr<const IGraph<V, W>> graph) override {
        return fbcgpu::exact_bc<W>(*graph, _o);
    }

  private:
    fbcgpu::Options _o;
};

template <typename V, typename W>
class GpuSSBrandesBC : public ISSBrandesBC<V, W> {
  public:
    explicit GpuSSBrandesBC(fbcgpu::Options o = {}) : _o(o) {}
    std::vector<W> singleSourceBrandes(V source, std::shared_ptr<const IGraph<V, W>> graph) override {
        auto d = _cache.get(graph, _o.device);
        return fbcgpu::single_source<W>(*d, (int32_t)source, _o);
    }

  private:
    fbcgpu::Options _o;
    fbcgpu::GraphCache _cache;
};

template <typename V, typename W>
class GpuClusterEvaluator : public IClusterEvaluator<V, W> {
  public:
    explicit GpuClusterEvaluator(fbcgpu::Options o = {}) : _o(o) {}
    void evaluateCluster(std::vector<W>& clusterBC,
                         std::vector<std::shared_ptr<VertexInfo<V, W>>>& globalVI,
                         std::shared_ptr<const ISubGraph<V, W>> cluster) override {
        auto d = _cache.get(cluster->referenceGraph(), _o.device);
        std::vector<std::vector<int32_t>> cv(1), bv(1);
        for (const V& v : cluster->vertices()) cv[0].push_back((int32_t)v);
        for (const V& b : cluster->borders()) bv[0].push_back((int32_t)b);
        std::vector<double> len;
        std::vector<uint64_t> cnt;
        std::vector<double> bc = fbcgpu::cluster_eval_batch(*d, cv, bv, _o, &len, &cnt, nullptr);
        const size_t nb = bv[0].size();
        std::lock_guard<std::mutex> lk(_out_mu);  // the reference calls this from OMP workers
        for (size_t i = 0; i < cv[0].size(); ++i) {
            const int32_t v = cv[0][i];
            clusterBC[v] += (W)bc[v];
            globalVI[v] = std::make_shared<VertexInfo<V, W>>((int)nb);
            for (size_t j = 0; j < nb; ++j) {
                globalVI[v]->setBorderSPLength((int)j, (W)len[i * nb + j]);
                globalVI[v]->setBorderSPCount((int)j, (V)(W)cnt[i * nb + j]);
            }
        }
    }

  private:
    fbcgpu::Options _o;
    fbcgpu::GraphCache _cache;
    std::mutex _out_mu;
};

template <typename V, typename W>
class GpuVertexInfoPivotSelector : public IPivotSelector<V, W> {
  public:
    explicit GpuVertexInfoPivotSelector(fbcgpu::Options o = {}) : _o(o) {}
    std::pair<std::vector<V>, std::vector<V>> selectPivots(const std::vector<W>& globalBC,
                                                           const std::vector<std::shared_ptr<VertexInfo<V, W>>>& verticesInfo,
                                                           const std::vector<V>& vertices,
                                                           const std::set<V>& borders) override {
        if (!fbcgpu::use_device_classes(verticesInfo, vertices, borders))
            return _host.selectPivots(globalBC, verticesInfo, vertices, borders);
#ifdef FASTBC_BRANDES_ENABLE_PIVOT_BORDER
        const bool pivot_border = true;
#else
        const bool pivot_border = false;
#endif
        std::lock_guard<std::mutex> lk(_mu);  // pivot selection may run on OpenMP workers
        return fbcgpu::select_pivots<V, W>(globalBC, verticesInfo, vertices, borders, pivot_border, _o.device);
    }

  private:
    fbcgpu::Options _o;
    VertexInfoPivotSelector<V, W> _host;
    std::mutex _mu;
};

template <typename V, typename W>
class GpuClusteredBrandesBC : public IBrandesBC<V, W> {
  public:
    GpuClusteredBrandesBC(std::shared_ptr<IGraphPartition<V, W>> gp,
                          std::shared_ptr<IPivotSelector<V, W>> ps, fbcgpu::Options o = {})
        : _gp(std::move(gp)), _ps(std::move(ps)), _o(o) {}

    std::vector<W> computeBC(const std::shared_ptr<const IGraph<V, W>> graph) override {
#ifdef FASTBC_BRANDES_CLUSTERED_IGNORE_UNCONNECTED
        const bool ignore_unconnected = true;
#else
        const bool ignore_unconnected = false;
#endif
        // the orchestration is fbcgpu::clustered_bc; the host parts are the reference's objects
        return fbcgpu::clustered_bc<V, W>(
            *graph,
            [&](const IGraph<V, W>&) {  // Louvain on the host (ClusteredBrandesBC.h:80-81)
                return _gp->partitionGraph(std::static_pointer_cast<const IDegreeGraph<V, W>>(graph));
            },
            [&](const std::vector<V>& community) {
                return std::shared_ptr<ISubGraph<V, W>>(std::make_shared<SubGraph<V, W>>(community, graph));
            },
            [](int nb) { return std::make_shared<VertexInfo<V, W>>(nb); },
            [&](const std::vector<W>& bc, const std::vector<std::shared_ptr<VertexInfo<V, W>>>& vi,
                const std::vector<V>& vertices, const std::set<V>& borders) {
                return _ps->selectPivots(bc, vi, vertices, borders);
            },
            _o, ignore_unconnected);
    }

  private:
    std::shared_ptr<IGraphPartition<V, W>> _gp;
    std::shared_ptr<IPivotSelector<V, W>> _ps;
    fbcgpu::Options _o;
};

}  // namespace brandes

namespace kmeans {

template <typename V, typename W>
class GpuPlusPlusKMeans : public IKMeans<V, W> {
  public:
    explicit GpuPlusPlusKMeans(fbcgpu::Options o = {}) : _o(o) {}
    std::pair<std::vector<V>, std::vector<V>> computeCentroids(
        int k, const std::vector<V>& vertices, const std::vector<V>& weights,
        const std::vector<std::shared_ptr<brandes::VertexInfo<V, W>>>& vertexInfo, W minVariance = 0,
        size_t maxIteration = 100) override {
        std::lock_guard<std::mutex> lk(_mu);  // pivot selection may run on OpenMP workers
        return fbcgpu::kmeans_centroids<V, W>(k, vertices, weights, vertexInfo, minVariance, maxIteration, _o.device);
    }

  private:
    fbcgpu::Options _o;
    std::mutex _mu;
};

}  // namespace kmeans

}  // namespace fastbc
