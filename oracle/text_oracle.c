/* Edge-list text reading in C -- TEST INFRASTRUCTURE ONLY (the checker and CPU baseline of
 * fbc_graph_from_text; the same rules as text_oracle.py, which states them with citations):
 * whitespace-separated triples "src dst weight" read as DirectedWeightedGraph(std::istream&)
 * does (DirectedWeightedGraph.h:67-96), then addEdge's merge of repeated pairs and the
 * ascending forward stars (DirectedWeightedGraph.h:136-170). */
#include <errno.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { ORC_TX_OK = 0, ORC_TX_WEIGHT = 1, ORC_TX_ID = 2, ORC_TX_INCOMPLETE = 3 };

static int tx_sp(unsigned char c) { return c == ' ' || (c >= 9 && c <= 13); }

/* next token of text[*pos, len): its start and length, or 0 at the end */
static int tx_next(const char* t, int64_t len, int64_t* pos, int64_t* start, int64_t* n) {
    int64_t p = *pos;
    while (p < len && tx_sp((unsigned char)t[p])) ++p;
    if (p >= len) {
        *pos = p;
        return 0;
    }
    *start = p;
    while (p < len && !tx_sp((unsigned char)t[p])) ++p;
    *n = p - *start;
    *pos = p;
    return 1;
}

static int tx_int(const char* s, int64_t n, int32_t* out) {
    int64_t k = 0, v = 0;
    int neg = 0;
    if (n > 0 && (s[0] == '+' || s[0] == '-')) {
        neg = s[0] == '-';
        k = 1;
    }
    if (k == n) return 0;
    for (; k < n; ++k) {
        if (s[k] < '0' || s[k] > '9') return 0;
        v = v * 10 + (s[k] - '0');
        if (v > 2147483648LL) return 0;
    }
    if (neg) v = -v;
    if (v > 2147483647LL) return 0;
    *out = (int32_t)v;
    return 1;
}

/* [+-]? (digits [. digits?] | . digits) ([eE] [+-]? digits)? over the whole token */
static int tx_dbl_form(const char* s, int64_t n) {
    int64_t k = 0, nd = 0;
    if (k < n && (s[k] == '+' || s[k] == '-')) ++k;
    while (k < n && s[k] >= '0' && s[k] <= '9') ++k, ++nd;
    if (k < n && s[k] == '.') {
        ++k;
        while (k < n && s[k] >= '0' && s[k] <= '9') ++k, ++nd;
    }
    if (nd == 0) return 0;
    if (k < n && (s[k] == 'e' || s[k] == 'E')) {
        int64_t ne = 0;
        ++k;
        if (k < n && (s[k] == '+' || s[k] == '-')) ++k;
        while (k < n && s[k] >= '0' && s[k] <= '9') ++k, ++ne;
        if (ne == 0) return 0;
    }
    return k == n;
}

/* Edges of the text into src/dst/w (capacity cap).  Returns ORC_TX_*; *count = edges read (the
 * reading ends before a weight that overflows a double); *edge = the offending edge index. */
int orc_parse_text(const char* t, int64_t len, int32_t* src, int32_t* dst, double* w, int64_t cap,
                   int64_t* count, int64_t* edge) {
    int64_t pos = 0, e = 0;
    char small[128];
    *count = 0;
    *edge = -1;
    for (;; ++e) {
        int64_t st[3], nn[3];
        int got = 0;
        while (got < 3 && tx_next(t, len, &pos, &st[got], &nn[got])) ++got;
        if (got == 0) break;
        if (got < 3) {
            *edge = e;
            return ORC_TX_INCOMPLETE;
        }
        int32_t a, b;
        if (!tx_int(t + st[0], nn[0], &a) || !tx_int(t + st[1], nn[1], &b)) {
            *edge = e;
            return ORC_TX_ID;
        }
        if (!tx_dbl_form(t + st[2], nn[2])) {
            *edge = e;
            return ORC_TX_WEIGHT;
        }
        char* buf = nn[2] < (int64_t)sizeof(small) ? small : (char*)malloc((size_t)nn[2] + 1);
        memcpy(buf, t + st[2], (size_t)nn[2]);
        buf[nn[2]] = 0;
        errno = 0;
        const double v = strtod(buf, NULL);
        if (buf != small) free(buf);
        if (v == HUGE_VAL) break; /* the reading ends before this edge */
        if (!(v > 0)) {
            *edge = e;
            return ORC_TX_WEIGHT;
        }
        if (e >= cap) {
            *edge = e;
            return -1;
        }
        src[e] = a;
        dst[e] = b;
        w[e] = v;
        *count = e + 1;
    }
    return ORC_TX_OK;
}

typedef struct {
    int32_t s, d;
    int64_t i;
} TxKey;

static int tx_cmp(const void* x, const void* y) {
    const TxKey* a = (const TxKey*)x;
    const TxKey* b = (const TxKey*)y;
    if (a->s != b->s) return a->s < b->s ? -1 : 1;
    if (a->d != b->d) return a->d < b->d ? -1 : 1;
    return a->i < b->i ? -1 : (a->i > b->i);
}

/* CSR over n vertices (n = 1 + the largest source, given by the caller): rows ascending by
 * destination, a repeated pair's weights summed in input order.  rp[n+1]; col, wout hold up to
 * m entries.  Returns the number of distinct pairs, or -1 when out of memory. */
int64_t orc_csr_from_edges(int64_t m, const int32_t* src, const int32_t* dst, const double* w, int32_t n,
                           int64_t* rp, int32_t* col, double* wout) {
    TxKey* k = (TxKey*)malloc(sizeof(TxKey) * (size_t)(m > 0 ? m : 1));
    if (!k) return -1;
    for (int64_t i = 0; i < m; ++i) {
        k[i].s = src[i];
        k[i].d = dst[i];
        k[i].i = i;
    }
    qsort(k, (size_t)m, sizeof(TxKey), tx_cmp);
    for (int32_t v = 0; v <= n; ++v) rp[v] = 0;
    int64_t out = 0;
    for (int64_t j = 0; j < m; ++j) {
        if (j > 0 && k[j].s == k[j - 1].s && k[j].d == k[j - 1].d) {
            wout[out - 1] += w[k[j].i];
        } else {
            col[out] = k[j].d;
            wout[out] = w[k[j].i];
            rp[k[j].s + 1]++;
            ++out;
        }
    }
    for (int32_t v = 0; v < n; ++v) rp[v + 1] += rp[v];
    free(k);
    return out;
}
