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
        const size_t n = graph->vertices().size();
        std::vector<W> globalBC(n, (W)0);
        std::vector<std::shared_ptr<VertexInfo<V, W>>> vi(n, nullptr);
        // Louvain on the host, as in the reference (ClusteredBrandesBC.h:80-81)
        auto communities = _gp->partitionGraph(std::static_pointer_cast<const IDegreeGraph<V, W>>(graph));
        std::vector<std::shared_ptr<ISubGraph<V, W>>> cl(communities.size());
        std::vector<size_t> evaluated;
        std::vector<std::vector<int32_t>> cv, bv;
        for (size_t i = 0; i < cl.size(); ++i) {
            cl[i] = std::make_shared<SubGraph<V, W>>(communities[i], graph);
#ifdef FASTBC_BRANDES_CLUSTERED_IGNORE_UNCONNECTED
            if (cl[i]->borders().empty()) continue;
#endif
            evaluated.push_back(i);
            cv.emplace_back();
            bv.emplace_back();
            for (const V& v : cl[i]->vertices()) cv.back().push_back((int32_t)v);
            for (const V& b : cl[i]->borders()) bv.back().push_back((int32_t)b);
        }
        auto d = fbcgpu::device_graph_for(*graph, _o.device);
        // every cluster's all-sources Brandes in one call (ClusteredBrandesBC.h:91-110)
        std::vector<double> len;
        std::vector<uint64_t> cnt;
        std::vector<int64_t> eo;
        std::vector<double> intra = fbcgpu::cluster_eval_batch(*d, cv, bv, _o, &len, &cnt, &eo);
        for (size_t k = 0; k < evaluated.size(); ++k) {
            const size_t nb = bv[k].size();
            for (size_t i = 0; i < cv[k].size(); ++i) {
                const int32_t v = cv[k][i];
                globalBC[v] += (W)intra[v];
                vi[v] = std::make_shared<VertexInfo<V, W>>((int)nb);
                for (size_t j = 0; j < nb; ++j) {
                    vi[v]->setBorderSPLength((int)j, (W)len[eo[k] + i * nb + j]);
                    vi[v]->setBorderSPCount((int)j, (V)(W)cnt[eo[k] + i * nb + j]);
                }
            }
        }
        // pivot selection on the host, in cluster order (ClusteredBrandesBC.h:112-114)
        std::vector<std::pair<std::vector<V>, std::vector<V>>> piv(cl.size());
        for (size_t i : evaluated)
            piv[i] = _ps->selectPivots(globalBC, vi, cl[i]->vertices(), cl[i]->borders());
        std::vector<W> intraClusterBC(globalBC);
        // every pivot's full-graph dependency in one call (ClusteredBrandesBC.h:141-155)
        std::vector<int32_t> pv;
        std::vector<double> cards;
        for (size_t c = 0; c < cl.size(); ++c)
            for (size_t p = 0; p < piv[c].first.size(); ++p) {
                pv.push_back((int32_t)piv[c].first[p]);
                cards.push_back((double)(W)piv[c].second[p]);
            }
        std::vector<double> acc(n, 0.0);
        if (!pv.empty()) fbcgpu::dependency_batch(*d, pv, cards, _o, acc);
        for (size_t v = 0; v < n; ++v) globalBC[v] += (W)acc[v];
        // duplicate intra-cluster dependency removed per pivot (ClusteredBrandesBC.h:158-164)
        for (size_t c = 0; c < cl.size(); ++c)
            for (size_t p = 0; p < piv[c].first.size(); ++p)
                for (const V& v : cl[c]->vertices())
                    globalBC[v] -= intraClusterBC[v] * (W)(piv[c].second[p]);
        return globalBC;
    }

  private:
    std::shared_ptr<IGraphPartition<V, W>> _gp;
    std::shared_ptr<IPivotSelector<V, W>> _ps;
    fbcgpu::Options _o;
};

}  // namespace brandes
}  // namespace fastbc
