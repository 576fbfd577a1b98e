/*
 * CPU oracle of the k-means step of the reference's pivot selection -- TEST INFRASTRUCTURE ONLY.
 *
 * Restates, for one cluster and one thread:
 *   PlusPlusKMeans::computeCentroids   libfastbc/include/kmeans/PlusPlusKMeans.h:76-147
 *   PlusPlusKMeans::_initPlusPlus      PlusPlusKMeans.h:150-183
 *   PlusPlusKMeans::_centroidVariance  PlusPlusKMeans.h:186-207
 *   KMeansPivotSelector::selectPivots  libfastbc/include/brandes/KMeansPivotSelector.h:79-132
 *                                      (k = max(floor(classes * kfrac), 1), duplicates removed)
 * over the exact classes' pivots (VertexInfoPivotSelector) and their border vectors, normalized
 * (lengths shifted by their minimum, VertexInfo.h:269-278).  VertexInfo::squaredDistance
 * (VertexInfo.h:295-308) sums (length difference)^2 + (count difference)^2 over the borders; between
 * two vertices every term is an integer, so the sum is exact in double whatever its order.  Against
 * a centroid (the members' mean, VertexInfo.h operator+= and operator/=) the terms are rounded and
 * the sum is taken in border order.  Products and sums are separately rounded (no fused
 * multiply-add: the Makefile builds the oracle with -ffp-contract=off).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "brandes_oracle.h"

/* squared distance of two vertices' vectors (exact: integer terms) */
static double sqd_vv(const double* la, const int32_t* ca, const double* lb, const int32_t* cb, int32_t b) {
    double s = 0.0;
    for (int32_t i = 0; i < b; ++i) {
        const double d = la[i] - lb[i];
        s += d * d;
        const double e = (double)(ca[i] - cb[i]);
        s += e * e;
    }
    return s;
}

/* squared distance of a centroid (means) and a vertex */
static double sqd_mv(const double* ml, const double* mc, const double* lb, const int32_t* cb, int32_t b) {
    double s = 0.0;
    for (int32_t i = 0; i < b; ++i) {
        const double d = ml[i] - lb[i];
        s += d * d;
        const double e = mc[i] - (double)cb[i];
        s += e * e;
    }
    return s;
}

int32_t orc_kmeans_pivots(int32_t np, int32_t b, const double* L, const int32_t* Cn, const int32_t* wt,
                          double kfrac, int32_t max_iter, int32_t* out_idx, int32_t* out_w) {
    if (np <= 0) return 0;
    int32_t k = (int32_t)((double)np * kfrac);
    if (k < 1) k = 1;
    const size_t bb = (size_t)(b > 0 ? b : 1);
    int32_t* cent = (int32_t*)malloc(sizeof(int32_t) * (size_t)k);
    int32_t* ncent = (int32_t*)malloc(sizeof(int32_t) * (size_t)k);
    double* cdist = (double*)calloc((size_t)np, sizeof(double));
    double* sl = (double*)malloc(sizeof(double) * (size_t)k * bb);
    double* sc = (double*)malloc(sizeof(double) * (size_t)k * bb);
    int32_t* cnt = (int32_t*)malloc(sizeof(int32_t) * (size_t)k);
    int32_t* first = (int32_t*)malloc(sizeof(int32_t) * (size_t)k);
    int32_t* last = (int32_t*)malloc(sizeof(int32_t) * (size_t)k);
    int32_t* next = (int32_t*)malloc(sizeof(int32_t) * (size_t)np);
    /* _initPlusPlus: the first pivot, then each time the vertex whose running mean distance to the
     * chosen centroids is largest (first on ties) */
    ncent[0] = 0;
    for (int32_t i = 1; i < k; ++i) {
        const int32_t lc = ncent[i - 1];
        const double p = 1.0 / i;
        const double q = 1.0 - p;
        int32_t far = 0;
        for (int32_t v = 0; v < np; ++v) {
            const double d = sqd_vv(L + (size_t)lc * b, Cn + (size_t)lc * b, L + (size_t)v * b, Cn + (size_t)v * b, b);
            cdist[v] = cdist[v] * q + d * p;
            if (cdist[v] > cdist[far]) far = v;
        }
        ncent[i] = far;
    }
    int32_t iter = 0;
    double var;
    do {
        ++iter;
        memcpy(cent, ncent, sizeof(int32_t) * (size_t)k);
        memset(sl, 0, sizeof(double) * (size_t)k * bb);
        memset(sc, 0, sizeof(double) * (size_t)k * bb);
        for (int32_t c = 0; c < k; ++c) { cnt[c] = 0; first[c] = -1; last[c] = -1; }
        /* each vertex to its nearest centroid (first on ties), summed in vertex order */
        for (int32_t v = 0; v < np; ++v) {
            const double* lv = L + (size_t)v * b;
            const int32_t* cv = Cn + (size_t)v * b;
            int32_t best = 0;
            double bd = sqd_vv(L + (size_t)cent[0] * b, Cn + (size_t)cent[0] * b, lv, cv, b);
            for (int32_t c = 1; c < k; ++c) {
                const double d = sqd_vv(L + (size_t)cent[c] * b, Cn + (size_t)cent[c] * b, lv, cv, b);
                if (d < bd) { bd = d; best = c; }
            }
            for (int32_t i = 0; i < b; ++i) {
                sl[(size_t)best * b + i] += lv[i];
                sc[(size_t)best * b + i] += (double)cv[i];
            }
            ++cnt[best];
            next[v] = -1;
            if (last[best] < 0) first[best] = v; else next[last[best]] = v;
            last[best] = v;
        }
        /* each centroid moves to its member nearest to the members' mean (first on ties) */
        for (int32_t c = 0; c < k; ++c) {
            ncent[c] = cent[c];
            if (!cnt[c]) continue;
            double* ml = sl + (size_t)c * b;
            double* mc = sc + (size_t)c * b;
            for (int32_t i = 0; i < b; ++i) {
                ml[i] /= (double)cnt[c];
                mc[i] /= (double)cnt[c];
            }
            int32_t bv = first[c];
            double bd = sqd_mv(ml, mc, L + (size_t)bv * b, Cn + (size_t)bv * b, b);
            for (int32_t v = next[bv]; v >= 0; v = next[v]) {
                const double d = sqd_mv(ml, mc, L + (size_t)v * b, Cn + (size_t)v * b, b);
                if (d < bd) { bd = d; bv = v; }
            }
            ncent[c] = bv;
        }
        var = 0.0;
        for (int32_t c = 0; c < k; ++c) {
            const double d = sqd_vv(L + (size_t)cent[c] * b, Cn + (size_t)cent[c] * b, L + (size_t)ncent[c] * b,
                                    Cn + (size_t)ncent[c] * b, b);
            if (d > var) var = d;
        }
    } while (var > 0.0 && iter <= max_iter);
    /* weights of the last assignment; a pivot chosen twice keeps its first entry */
    int32_t out = 0;
    for (int32_t c = 0; c < k; ++c) {
        int32_t wsum = 0;
        for (int32_t v = first[c]; v >= 0; v = next[v]) wsum += wt[v];
        int dup = 0;
        for (int32_t j = 0; j < out && !dup; ++j) dup = out_idx[j] == cent[c];
        if (dup) continue;
        out_idx[out] = cent[c];
        out_w[out] = wsum;
        ++out;
    }
    free(cent); free(ncent); free(cdist); free(sl); free(sc); free(cnt); free(first); free(last);
    free(next);
    return out;
}
