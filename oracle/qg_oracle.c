/*
 * qg_oracle.c -- CPU oracle for the relational-operator hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
 * compared against (tests/, __graft_entry__.smoke(), and the cpu_baseline /
 * --impl reference legs of bench.py).  Nothing in the product library links,
 * loads or calls it.
 *
 * It is a plain-C restatement of the reference operators' semantics
 * (Xtra-Computing/Query_on_OpenCL_FPGA); every function names the reference
 * file:line it follows.  Record = uint2 {x, y}: y is the key, x the payload /
 * row id (host/host/common.h:27-28).
 *
 * Parity pin: the generator, filter, scan, sort and group-by restatements are
 * checked against the reference's own generator and validators compiled from
 * the reference sources (oracle/build_ref.sh) and against golden vectors made
 * from them (tests/golden/make_golden.py).
 *
 * Multi-threaded variants (OpenMP) are used only to time the CPU baseline; they
 * produce the same results as the scalar forms.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_EXPORT __attribute__((visibility("default")))

ORC_EXPORT int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

ORC_EXPORT void orc_set_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

/* ------------------------------------------------------------------------ */
/* Generators                                                                */
/* ------------------------------------------------------------------------ */

/* host/host/generator.cpp:63-77 (generateRand).  The reference draws four
 * rand() values per record; under glibc RAND_MAX is 2^31-1, so `rand()<<1`
 * wraps in 32-bit int arithmetic and keys can be negative.  The draws are
 * evaluated in the order gcc evaluates the reference expression (checked by
 * tests/test_oracle_pins.py against the reference compiled here). */
ORC_EXPORT void orc_generate_rand(uint32_t *R, int maxmax, int64_t n, int seed) {
    const uint32_t offset = (1u << 15) - 1;
    srand((unsigned)seed);
    for (int64_t i = 0; i < n; i++) {
        uint32_t a = (uint32_t)rand();
        uint32_t b = (uint32_t)rand();
        uint32_t c = (uint32_t)rand();
        uint32_t d = (uint32_t)rand();
        uint32_t v = ((a & offset) << 15) + (b & 1u) + (c << 1) + (d & 1u);
        int32_t s = (int32_t)v;
        R[2 * i + 1] = (uint32_t)(s % maxmax);
        R[2 * i + 0] = (uint32_t)i;
    }
}

/* host/host/generator.cpp:82-93 (generateRandInt) */
ORC_EXPORT void orc_generate_rand_int(int32_t *R, int maxv, int64_t n, int seed) {
    const uint32_t offset = (1u << 15) - 1;
    srand((unsigned)seed);
    for (int64_t i = 0; i < n; i++) {
        uint32_t a = (uint32_t)rand();
        uint32_t b = (uint32_t)rand();
        uint32_t c = (uint32_t)rand();
        uint32_t d = (uint32_t)rand();
        uint32_t v = ((a & offset) << 15) + (b & 1u) + (c << 1) + (d & 1u);
        R[i] = ((int32_t)v) % maxv;
    }
}

/* ------------------------------------------------------------------------ */
/* Filter                                                                    */
/* ------------------------------------------------------------------------ */

/* kernel/filter/filter_op.cl:6-31 (map: signed inclusive range on .y),
 * :220-238 (stable scatter), host/host/Validate.cpp:317-370 (positional
 * compare).  Returns the number of selected records. */
ORC_EXPORT int64_t orc_filter_rec(const uint32_t *in, int64_t n, int32_t lo, int32_t hi,
                                  uint32_t *out) {
    int64_t k = 0;
    for (int64_t i = 0; i < n; i++) {
        int32_t key = (int32_t)in[2 * i + 1];
        if (key >= lo && key <= hi) {
            out[2 * k] = in[2 * i];
            out[2 * k + 1] = in[2 * i + 1];
            k++;
        }
    }
    return k;
}

/* Column form of the same operator (config 0): predicate lo <= key <= hi on an
 * int32 key column; output (row_id, payload) int32 pairs in input order. */
ORC_EXPORT int64_t orc_filter_cols(const int32_t *key, const int32_t *pay, int64_t n,
                                   int32_t lo, int32_t hi, int32_t *out_pairs) {
    int64_t k = 0;
    for (int64_t i = 0; i < n; i++) {
        if (key[i] >= lo && key[i] <= hi) {
            out_pairs[2 * k] = (int32_t)i;
            out_pairs[2 * k + 1] = pay[i];
            k++;
        }
    }
    return k;
}

/* Multi-threaded column filter (CPU baseline): per-thread count, exclusive
 * prefix over threads, then stable per-thread write. */
ORC_EXPORT int64_t orc_filter_cols_mt(const int32_t *key, const int32_t *pay, int64_t n,
                                      int32_t lo, int32_t hi, int32_t *out_pairs) {
    int nt = orc_num_threads();
    int64_t *cnt = (int64_t *)calloc((size_t)nt + 1, sizeof(int64_t));
    int64_t total = 0;
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
#else
        int t = 0;
#endif
        int64_t b = n * t / nt, e = n * (t + 1) / nt, c = 0;
        for (int64_t i = b; i < e; i++) c += (key[i] >= lo) & (key[i] <= hi);
        cnt[t + 1] = c;
#pragma omp barrier
#pragma omp single
        {
            for (int j = 0; j < nt; j++) cnt[j + 1] += cnt[j];
            total = cnt[nt];
        }
        int64_t k = cnt[t];
        for (int64_t i = b; i < e; i++) {
            if (key[i] >= lo && key[i] <= hi) {
                out_pairs[2 * k] = (int32_t)i;
                out_pairs[2 * k + 1] = pay[i];
                k++;
            }
        }
    }
    free(cnt);
    return total;
}

/* ------------------------------------------------------------------------ */
/* Scan                                                                      */
/* ------------------------------------------------------------------------ */

/* host/host/Validate.cpp:4-37 (validateScan): exclusive int32 prefix sum with
 * two's-complement wrap (the kernels add in int, filter_op.cl:51-207). */
ORC_EXPORT void orc_scan_excl_i32(const int32_t *in, int64_t n, int32_t *out) {
    uint32_t acc = 0;
    for (int64_t i = 0; i < n; i++) {
        out[i] = (int32_t)acc;
        acc += (uint32_t)in[i];
    }
}

/* ------------------------------------------------------------------------ */
/* Sort                                                                      */
/* ------------------------------------------------------------------------ */

/* Ascending sort of records by .y as unsigned (bitonicSortShared /
 * bitonicMergeGlobal compare `aa.y > bb.y` on uint,
 * kernel/aggregation/1/group_by_cu_op_dp.cl:132, 186-284).  The reference sort
 * is not stable; this restatement is a stable LSD radix sort, so tests compare
 * the payload order within equal keys as a multiset. */
ORC_EXPORT void orc_sort_rec_by_y(uint32_t *R, int64_t n) {
    if (n <= 1) return;
    uint64_t *a = (uint64_t *)malloc((size_t)n * 8), *b = (uint64_t *)malloc((size_t)n * 8);
    for (int64_t i = 0; i < n; i++) a[i] = ((uint64_t)R[2 * i + 1] << 32) | R[2 * i];
    for (int pass = 0; pass < 4; pass++) {
        int shift = 32 + 8 * pass;
        int64_t cnt[257] = {0};
        for (int64_t i = 0; i < n; i++) cnt[((a[i] >> shift) & 255) + 1]++;
        for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
        for (int64_t i = 0; i < n; i++) b[cnt[(a[i] >> shift) & 255]++] = a[i];
        uint64_t *t = a; a = b; b = t;
    }
    for (int64_t i = 0; i < n; i++) {
        R[2 * i] = (uint32_t)a[i];
        R[2 * i + 1] = (uint32_t)(a[i] >> 32);
    }
    free(a);
    free(b);
}

/* ------------------------------------------------------------------------ */
/* Group-by on sorted records: labels, numGroups, startPos                   */
/* ------------------------------------------------------------------------ */

/* kernel/aggregation/1/group_by_cu_op_dp.cl:293-327 (scanGroupLabel: label[0]=1,
 * label[i+1] = key[i] != key[i+1]), :505-509 (numGroups = label[n-1] +
 * scan[n-1]), :511-528 (startPos[scan[i]] = i where label[i]);
 * host/host/testGroupBy.cpp:81-154.  `sorted` must already be sorted by .y.
 * Returns numGroups; startPos needs room for numGroups entries. */
ORC_EXPORT int64_t orc_group_startpos(const uint32_t *sorted, int64_t n, int32_t *startPos) {
    if (n <= 0) return 0;
    int64_t g = 0;
    startPos[g++] = 0;
    for (int64_t i = 1; i < n; i++)
        if ((int32_t)sorted[2 * i + 1] != (int32_t)sorted[2 * (i - 1) + 1]) startPos[g++] = (int32_t)i;
    return g;
}

/* kernel/aggregation/1/group_by_cu_op_dp.cl:547-716 (parallelAggregate_kernel)
 * over .x of group g = rows [startPos[g], startPos[g+1] or n):
 *   op 0 SUM : int32 sum with wrap
 *   op 1 MAX : signed max, initial value 0 (:560-571)
 *   op 2 MIN : signed min, initial value 1<<30 (TEST_MAX, :14, :563-564)
 *   op 3 AVG : wrapped int32 sum / (end-start), C division (:705-707) */
ORC_EXPORT void orc_aggregate_groups(const uint32_t *sorted, int64_t n, const int32_t *startPos,
                                     int64_t numGroups, int op, int32_t *agg) {
    for (int64_t g = 0; g < numGroups; g++) {
        int64_t s = startPos[g], e = (g == numGroups - 1) ? n : startPos[g + 1];
        int32_t acc = (op == 2) ? (1 << 30) : 0;
        uint32_t sum = 0;
        for (int64_t i = s; i < e; i++) {
            int32_t v = (int32_t)sorted[2 * i];
            if (op == 1) { if (v > acc) acc = v; }
            else if (op == 2) { if (v < acc) acc = v; }
            else sum += (uint32_t)v;
        }
        if (op == 0) acc = (int32_t)sum;
        if (op == 3) acc = (e > s) ? ((int32_t)sum) / (int32_t)(e - s) : 0;
        agg[g] = acc;
    }
}

/* ------------------------------------------------------------------------ */
/* Column group-by with int64 SUM + COUNT (configs 1 and 1-fused)            */
/* ------------------------------------------------------------------------ */

/* The group-by + aggregate chain (testAggAfterGB.cpp:127-255 over
 * group_by_cu_op_dp.cl) with the aggregate widened to int64 SUM plus COUNT and
 * an optional row predicate lo2 <= val2 <= hi2 applied first (the fused
 * filter_aggregation image, kernel/filter_aggregation/
 * filter_aggregation_cu_op_dp.cl:82-139 then :151-778).  Output groups are in
 * ascending unsigned key order, the order groupByImpl's sorted array gives.
 * Returns numGroups, or -1 if more than `cap` groups exist. */
static int cmp_u32(const void *a, const void *b) {
    uint32_t x = *(const uint32_t *)a, y = *(const uint32_t *)b;
    return (x > y) - (x < y);
}

typedef struct { uint32_t key; int32_t used; int64_t sum; int64_t cnt; } orc_slot;

static uint32_t orc_hash32(uint32_t k) {
    k ^= k >> 16; k *= 0x7feb352dU; k ^= k >> 15; k *= 0x846ca68bU; k ^= k >> 16;
    return k;
}

static int64_t orc_groupby_core(const int32_t *key, const int32_t *val, const int32_t *val2,
                                int32_t lo2, int32_t hi2, int64_t b, int64_t e,
                                orc_slot *tab, uint64_t mask) {
    int64_t used = 0;
    for (int64_t i = b; i < e; i++) {
        if (val2 && !(val2[i] >= lo2 && val2[i] <= hi2)) continue;
        uint32_t k = (uint32_t)key[i];
        uint64_t h = orc_hash32(k) & mask;
        while (tab[h].used && tab[h].key != k) h = (h + 1) & mask;
        if (!tab[h].used) { tab[h].used = 1; tab[h].key = k; used++; }
        tab[h].sum += val[i];
        tab[h].cnt += 1;
    }
    return used;
}

static int64_t orc_emit_sorted(orc_slot *tab, uint64_t cap_tab, int64_t cap, int32_t *gkey,
                               int64_t *gsum, int64_t *gcnt) {
    int64_t g = 0;
    for (uint64_t s = 0; s < cap_tab; s++) if (tab[s].used) g++;
    if (g > cap) return -1;
    uint32_t *keys = (uint32_t *)malloc((size_t)(g ? g : 1) * 4);
    int64_t j = 0;
    for (uint64_t s = 0; s < cap_tab; s++) if (tab[s].used) keys[j++] = tab[s].key;
    qsort(keys, (size_t)g, 4, cmp_u32);
    uint64_t mask = cap_tab - 1;
    for (int64_t i = 0; i < g; i++) {
        uint32_t k = keys[i];
        uint64_t h = orc_hash32(k) & mask;
        while (tab[h].key != k || !tab[h].used) h = (h + 1) & mask;
        gkey[i] = (int32_t)k; gsum[i] = tab[h].sum; gcnt[i] = tab[h].cnt;
    }
    free(keys);
    return g;
}

static uint64_t orc_pow2_at_least(uint64_t v) {
    uint64_t c = 16;
    while (c < v) c <<= 1;
    return c;
}

ORC_EXPORT int64_t orc_groupby_cols(const int32_t *key, const int32_t *val, const int32_t *val2,
                                    int32_t lo2, int32_t hi2, int64_t n, int64_t cap,
                                    int32_t *gkey, int64_t *gsum, int64_t *gcnt) {
    uint64_t ct = orc_pow2_at_least((uint64_t)(n < cap ? n : cap) * 2 + 2);
    orc_slot *tab = (orc_slot *)calloc(ct, sizeof(orc_slot));
    orc_groupby_core(key, val, val2, lo2, hi2, 0, n, tab, ct - 1);
    int64_t g = orc_emit_sorted(tab, ct, cap, gkey, gsum, gcnt);
    free(tab);
    return g;
}

/* Multi-threaded form (CPU baseline): per-thread tables merged serially. */
ORC_EXPORT int64_t orc_groupby_cols_mt(const int32_t *key, const int32_t *val, const int32_t *val2,
                                       int32_t lo2, int32_t hi2, int64_t n, int64_t cap,
                                       int32_t *gkey, int64_t *gsum, int64_t *gcnt) {
    int nt = orc_num_threads();
    uint64_t ct = orc_pow2_at_least((uint64_t)(n < cap ? n : cap) * 2 + 2);
    orc_slot **tabs = (orc_slot **)calloc((size_t)nt, sizeof(orc_slot *));
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        int t = omp_get_thread_num();
#else
        int t = 0;
#endif
        int64_t b = n * t / nt, e = n * (t + 1) / nt;
        uint64_t need = orc_pow2_at_least((uint64_t)(e - b < cap ? e - b : cap) * 2 + 2);
        (void)need;
        tabs[t] = (orc_slot *)calloc(ct, sizeof(orc_slot));
        orc_groupby_core(key, val, val2, lo2, hi2, b, e, tabs[t], ct - 1);
    }
    orc_slot *tab = tabs[0];
    uint64_t mask = ct - 1;
    for (int t = 1; t < nt; t++) {
        for (uint64_t s = 0; s < ct; s++) {
            if (!tabs[t][s].used) continue;
            uint32_t k = tabs[t][s].key;
            uint64_t h = orc_hash32(k) & mask;
            while (tab[h].used && tab[h].key != k) h = (h + 1) & mask;
            if (!tab[h].used) { tab[h].used = 1; tab[h].key = k; }
            tab[h].sum += tabs[t][s].sum;
            tab[h].cnt += tabs[t][s].cnt;
        }
        free(tabs[t]);
    }
    int64_t g = orc_emit_sorted(tab, ct, cap, gkey, gsum, gcnt);
    free(tab);
    free(tabs);
    return g;
}

/* ------------------------------------------------------------------------ */
/* Hash join + filter + sort (config 2)                                      */
/* ------------------------------------------------------------------------ */

/* kernel/hj_filter_sort/1/hj_filter_sort_op.cl:25-60 (build: every R tuple is
 * stored), :62-109 (probe: every R tuple whose uint key equals the S key is a
 * match, all matches emitted), then the filter (:117-349) and sort by key
 * (:362-564).  Config 2 filters S.payload before the join; the output is
 * (key, R.payload, S.payload) sorted by key.  Equal-key rows come out in
 * ascending (R.payload, S.payload) order here; the GPU's order among equal
 * keys is unspecified, so tests compare per-key multisets.  Returns the row
 * count, or -(needed) - 1 if it exceeds cap. */
typedef struct { uint32_t key; uint32_t rpay; uint32_t spay; } orc_jrow;

static int cmp_jrow(const void *a, const void *b) {
    const orc_jrow *x = (const orc_jrow *)a, *y = (const orc_jrow *)b;
    if (x->key != y->key) return (x->key > y->key) - (x->key < y->key);
    if (x->rpay != y->rpay) return ((int32_t)x->rpay > (int32_t)y->rpay) - ((int32_t)x->rpay < (int32_t)y->rpay);
    return ((int32_t)x->spay > (int32_t)y->spay) - ((int32_t)x->spay < (int32_t)y->spay);
}

typedef struct { int64_t *head; int64_t *next; uint64_t mask; } orc_jtab;

static void orc_jtab_build(orc_jtab *t, const int32_t *rkey, int64_t nR) {
    uint64_t ct = orc_pow2_at_least((uint64_t)nR * 2 + 2);
    t->mask = ct - 1;
    t->head = (int64_t *)malloc(ct * sizeof(int64_t));
    t->next = (int64_t *)malloc((size_t)(nR ? nR : 1) * sizeof(int64_t));
    for (uint64_t i = 0; i < ct; i++) t->head[i] = -1;
    for (int64_t i = 0; i < nR; i++) {
        uint64_t h = orc_hash32((uint32_t)rkey[i]) & t->mask;
        t->next[i] = t->head[h];
        t->head[h] = i;
    }
}

static void orc_jtab_free(orc_jtab *t) { free(t->head); free(t->next); }

ORC_EXPORT int64_t orc_join_filter_sort(const int32_t *rkey, const int32_t *rpay, int64_t nR,
                                        const int32_t *skey, const int32_t *spay, int64_t nS,
                                        int32_t slo, int32_t shi, int64_t cap,
                                        int32_t *okey, int32_t *orpay, int32_t *ospay) {
    orc_jtab t;
    orc_jtab_build(&t, rkey, nR);
    int64_t cnt = 0;
    for (int64_t i = 0; i < nS; i++) {
        if (!(spay[i] >= slo && spay[i] <= shi)) continue;
        uint32_t k = (uint32_t)skey[i];
        for (int64_t j = t.head[orc_hash32(k) & t.mask]; j >= 0; j = t.next[j])
            if ((uint32_t)rkey[j] == k) cnt++;
    }
    if (cnt > cap) { orc_jtab_free(&t); return -cnt - 1; }
    orc_jrow *rows = (orc_jrow *)malloc((size_t)(cnt ? cnt : 1) * sizeof(orc_jrow));
    int64_t m = 0;
    for (int64_t i = 0; i < nS; i++) {
        if (!(spay[i] >= slo && spay[i] <= shi)) continue;
        uint32_t k = (uint32_t)skey[i];
        for (int64_t j = t.head[orc_hash32(k) & t.mask]; j >= 0; j = t.next[j])
            if ((uint32_t)rkey[j] == k) {
                rows[m].key = k; rows[m].rpay = (uint32_t)rpay[j]; rows[m].spay = (uint32_t)spay[i];
                m++;
            }
    }
    qsort(rows, (size_t)m, sizeof(orc_jrow), cmp_jrow);
    for (int64_t i = 0; i < m; i++) {
        okey[i] = (int32_t)rows[i].key; orpay[i] = (int32_t)rows[i].rpay; ospay[i] = (int32_t)rows[i].spay;
    }
    free(rows);
    orc_jtab_free(&t);
    return m;
}

/* Multi-threaded form (CPU baseline): serial build, parallel probe into
 * per-thread buffers, per-thread radix sort by key, k-way merge by thread. */
static void orc_radix_jrows(orc_jrow *a, orc_jrow *b, int64_t n) {
    for (int pass = 0; pass < 4; pass++) {
        int shift = 8 * pass;
        int64_t c[257] = {0};
        for (int64_t i = 0; i < n; i++) c[((a[i].key >> shift) & 255) + 1]++;
        if (c[((a[0].key >> shift) & 255) + 1] == n) continue;
        for (int d = 0; d < 256; d++) c[d + 1] += c[d];
        for (int64_t i = 0; i < n; i++) b[c[(a[i].key >> shift) & 255]++] = a[i];
        memcpy(a, b, (size_t)n * sizeof(orc_jrow));
    }
}

ORC_EXPORT int64_t orc_join_filter_sort_mt(const int32_t *rkey, const int32_t *rpay, int64_t nR,
                                           const int32_t *skey, const int32_t *spay, int64_t nS,
                                           int32_t slo, int32_t shi, int64_t cap,
                                           int32_t *okey, int32_t *orpay, int32_t *ospay) {
    orc_jtab t;
    orc_jtab_build(&t, rkey, nR);
    int nt = orc_num_threads();
    orc_jrow **buf = (orc_jrow **)calloc((size_t)nt, sizeof(orc_jrow *));
    int64_t *cnt = (int64_t *)calloc((size_t)nt + 1, sizeof(int64_t));
    int over = 0;
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
        int th = omp_get_thread_num();
#else
        int th = 0;
#endif
        int64_t b = nS * th / nt, e = nS * (th + 1) / nt, m = 0, room = 1024;
        orc_jrow *rows = (orc_jrow *)malloc((size_t)room * sizeof(orc_jrow));
        for (int64_t i = b; i < e; i++) {
            if (!(spay[i] >= slo && spay[i] <= shi)) continue;
            uint32_t k = (uint32_t)skey[i];
            for (int64_t j = t.head[orc_hash32(k) & t.mask]; j >= 0; j = t.next[j])
                if ((uint32_t)rkey[j] == k) {
                    if (m == room) { room *= 2; rows = (orc_jrow *)realloc(rows, (size_t)room * sizeof(orc_jrow)); }
                    rows[m].key = k; rows[m].rpay = (uint32_t)rpay[j]; rows[m].spay = (uint32_t)spay[i];
                    m++;
                }
        }
        if (m > 0) {
            orc_jrow *tmp = (orc_jrow *)malloc((size_t)m * sizeof(orc_jrow));
            orc_radix_jrows(rows, tmp, m);
            free(tmp);
        }
        buf[th] = rows;
        cnt[th + 1] = m;
    }
    int64_t total = 0;
    for (int th = 0; th < nt; th++) total += cnt[th + 1];
    if (total > cap) over = 1;
    if (!over) {
        int64_t *pos = (int64_t *)calloc((size_t)nt, sizeof(int64_t));
        for (int64_t o = 0; o < total; o++) {
            int best = -1;
            for (int th = 0; th < nt; th++)
                if (pos[th] < cnt[th + 1] && (best < 0 || buf[th][pos[th]].key < buf[best][pos[best]].key)) best = th;
            orc_jrow r = buf[best][pos[best]++];
            okey[o] = (int32_t)r.key; orpay[o] = (int32_t)r.rpay; ospay[o] = (int32_t)r.spay;
        }
        free(pos);
    }
    for (int th = 0; th < nt; th++) free(buf[th]);
    free(buf); free(cnt);
    orc_jtab_free(&t);
    return over ? -total - 1 : total;
}

/* Reference-layout hash build + probe (hj_filter_sort_op.cl:25-109): R and S
 * are interleaved uint (key, val) pairs; every match emits (S.val, R.val).
 * The reference leaves holes in a per-work-item output region; this form is
 * compacted, in S order and, per S row, in R order.  Returns the match count,
 * or -(needed)-1 if it exceeds cap. */
ORC_EXPORT int64_t orc_hash_join_ref(const uint32_t *r, int64_t nR, const uint32_t *s, int64_t nS,
                                     int64_t cap, uint32_t *out) {
    int32_t *rk = (int32_t *)malloc((size_t)(nR ? nR : 1) * 4);
    for (int64_t i = 0; i < nR; i++) rk[i] = (int32_t)r[2 * i];
    orc_jtab t;
    orc_jtab_build(&t, rk, nR);
    int64_t m = 0;
    for (int64_t i = 0; i < nS; i++) {
        uint32_t k = s[2 * i];
        /* chain is in reverse insertion order; emit in R order */
        int64_t hits[64]; int nh = 0;
        for (int64_t j = t.head[orc_hash32(k) & t.mask]; j >= 0; j = t.next[j]) {
            if (r[2 * j] != k) continue;
            if (nh < 64) hits[nh++] = j;
            else { if (m < cap) { out[2 * m] = s[2 * i + 1]; out[2 * m + 1] = r[2 * j + 1]; } m++; }
        }
        for (int q = nh - 1; q >= 0; q--) {
            if (m < cap) { out[2 * m] = s[2 * i + 1]; out[2 * m + 1] = r[2 * hits[q] + 1]; }
            m++;
        }
    }
    orc_jtab_free(&t);
    free(rk);
    return m > cap ? -m - 1 : m;
}

/* ---- learned cost model (no reference counterpart: the reference's cost
 * model is the static table of host/dynamic_programming.cpp:152-167) ----
 * Restatement of the 16 -> 64 (ReLU) -> 1 MLP of csrc/qg_mlp.cu in double
 * precision, the checker of the GPU forward pass and gradients.
 * Parameters: W1[64][16], b1[64], W2[64], b2. */
#define ORC_MI 16
#define ORC_MH 64
ORC_EXPORT void orc_mlp_forward(const float *p, const float *X, int64_t n, double *out) {
    const float *W1 = p, *b1 = p + ORC_MI * ORC_MH, *W2 = b1 + ORC_MH, *b2 = W2 + ORC_MH;
    for (int64_t s = 0; s < n; s++) {
        double o = b2[0];
        for (int j = 0; j < ORC_MH; j++) {
            double a = b1[j];
            for (int k = 0; k < ORC_MI; k++) a += (double)W1[j * ORC_MI + k] * X[s * ORC_MI + k];
            if (a > 0) o += a * W2[j];
        }
        out[s] = o;
    }
}

/* Gradient of mean((f(x) - y)^2); returns the loss. */
ORC_EXPORT double orc_mlp_grad(const float *p, const float *X, const float *y, int64_t n, double *grad) {
    const float *W1 = p, *b1 = p + ORC_MI * ORC_MH, *W2 = b1 + ORC_MH, *b2 = W2 + ORC_MH;
    const int P = ORC_MI * ORC_MH + 2 * ORC_MH + 1;
    for (int q = 0; q < P; q++) grad[q] = 0;
    double loss = 0, z[ORC_MH];
    for (int64_t s = 0; s < n; s++) {
        double o = b2[0];
        for (int j = 0; j < ORC_MH; j++) {
            double a = b1[j];
            for (int k = 0; k < ORC_MI; k++) a += (double)W1[j * ORC_MI + k] * X[s * ORC_MI + k];
            z[j] = a;
            if (a > 0) o += a * W2[j];
        }
        const double d = o - y[s];
        loss += d * d;
        const double go = 2.0 * d / (double)n;
        grad[P - 1] += go;
        for (int j = 0; j < ORC_MH; j++) {
            if (z[j] <= 0) continue;
            grad[ORC_MI * ORC_MH + ORC_MH + j] += go * z[j];
            const double gz = go * W2[j];
            grad[ORC_MI * ORC_MH + j] += gz;
            for (int k = 0; k < ORC_MI; k++) grad[j * ORC_MI + k] += gz * X[s * ORC_MI + k];
        }
    }
    return loss / (double)n;
}

/* Whole-column reduce of Record.y as host/host/Validate.cpp:372-468 checks it:
 * unsigned y, SUM wraps modulo 2^32, MAX/MIN compare unsigned (int
 * accumulator promoted), AVERAGE = wrapped sum / n.  n >= 1. */
ORC_EXPORT uint32_t orc_reduce_rec(const uint32_t *rec, int64_t n, int op) {
    uint32_t acc = rec[1];
    if (op == 0 || op == 3) {
        acc = 0;
        for (int64_t i = 0; i < n; i++) acc += rec[2 * i + 1];
        if (op == 3) acc = acc / (uint32_t)n;
        return acc;
    }
    for (int64_t i = 1; i < n; i++) {
        uint32_t y = rec[2 * i + 1];
        if (op == 1 ? y > acc : y < acc) acc = y;
    }
    return acc;
}

/* Radix split (host/host/testSplit.cpp:156-209; its map kernel is not
 * shipped): stable counting partition by y mod parts; bound[p] = first row. */
ORC_EXPORT void orc_split_rec(const uint32_t *rec, int64_t n, int32_t parts, uint32_t *out, int32_t *bound) {
    int64_t *cnt = (int64_t *)calloc((size_t)parts + 1, sizeof(int64_t));
    for (int64_t i = 0; i < n; i++) cnt[rec[2 * i + 1] % (uint32_t)parts + 1]++;
    for (int32_t p = 0; p < parts; p++) cnt[p + 1] += cnt[p];
    for (int32_t p = 0; p < parts; p++) bound[p] = (int32_t)cnt[p];
    for (int64_t i = 0; i < n; i++) {
        int64_t o = cnt[rec[2 * i + 1] % (uint32_t)parts]++;
        out[2 * o] = rec[2 * i];
        out[2 * o + 1] = rec[2 * i + 1];
    }
    free(cnt);
}
