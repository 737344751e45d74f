/*
 * pfp_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C, CPU restatement of the reference's prefix-free-parsing (PFP)
 * BWT construction, written stage by stage so that every intermediate of the
 * reference (phrase ends D, phrase meta-characters, parse suffix array,
 * colex order, the suffix set S, colex intervals, run / mixed blocks) can be
 * compared with the GPU path.  Only tests/, __graft_entry__.smoke() and the
 * CPU legs of bench.py may load this file's library; it is never part of the
 * product path.
 *
 * Parity anchor.  The reference ships no golden vectors; its only
 * correctness check is a byte-for-byte `cmp` of the PFP output against
 * libcubwt's output (compare_script.sh:7-10).  This oracle is therefore
 * pinned against an independent suffix-array BWT in the output convention
 * of libcubwt's harness (sa_bwt.c, libcubwt.cu:2242-2254 and
 * libcubwt.cu:2989-3020), on every test input.  The reference binaries
 * themselves are CUDA programs that could not be executed where this file
 * was written, so the restatement is not pinned against their outputs.
 *
 * Citations use the file names of the reference project; "K" below is
 * Prefix_Free_Parsing_W=5_P=16_kommentiert.cu.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

/* ------------------------------------------------------------------ */
/* Stage 0: input contract, K:111-150 (Scan_input).                     */
/* Text bytes must lie in [2,254]; W copies of byte 1 are appended.     */
/* ------------------------------------------------------------------ */
int gbo_validate(const uint8_t *T, int64_t n, int small_alphabet)
{
    /* Any byte outside [2,254] is a bad parameter (the reference asserts);
     * with the small-alphabet flag a byte in [16,254] is outside the range
     * its digit packing handles (..._small_alphabet.cu:995-1002). */
    int64_t i;
    int small_bad = 0;
    for (i = 0; i < n; i++) {
        if (T[i] < 2 || T[i] == 255) return GBO_BAD_PARAMETER;
        if (T[i] > 15) small_bad = 1;
    }
    return (small_alphabet && small_bad) ? GBO_UNSUPPORTED_INPUT : 0;
}

/* X = T . 1^W  (K:146-149) */
static uint8_t *make_enlarged(const uint8_t *T, int64_t n, int W)
{
    uint8_t *X = (uint8_t *)malloc((size_t)(n + W + 1));
    if (!X) return NULL;
    memcpy(X, T, (size_t)n);
    memset(X + n, 1, (size_t)W);
    X[n + W] = 0;
    return X;
}

/* ------------------------------------------------------------------ */
/* Stage 1: trigger scan, K:443-576 (Compute_D1/D2/D3).                 */
/* Window s (s+W-1 < n) is a trigger when its hash                       */
/*   h = sum_{k<W} T[s+W-1-k] * (2^k mod P)  (mod P)                    */
/* is 0, or when T[s..s+W-1] == T[0..W-1]; window 0 never triggers.      */
/* D receives the window's last position; n+W-1 is appended last.        */
/* D needs room for max(n-W+1,0)+1 entries.  Returns z = |D|.           */
/* ------------------------------------------------------------------ */
static int is_trigger(const uint8_t *T, int64_t s, int W, int P)
{
    int pot = 1, res = 0, equal = 1, i;
    for (i = W - 1; i >= 0; i--) {                  /* K:468-473 */
        if (equal && T[s + i] != T[i]) equal = 0;
        res = (res + pot * (int)T[s + i]) % P;
        pot = (pot * 2) % P;
    }
    return s > 0 && (res == 0 || equal);            /* K:475 */
}

int64_t gbo_trigger_scan(const uint8_t *T, int64_t n, int W, int P, int64_t *D)
{
    const int64_t nw = n - W + 1 > 0 ? n - W + 1 : 0;    /* windows s with s+W-1 < n */
    int64_t z = 0, s;
#ifdef _OPENMP
    if (nw > (1 << 20)) {
        /* windows are independent: count per chunk, then write at the chunk's offset */
        extern int omp_get_max_threads(void);
        const int64_t nch = 8 * (int64_t)omp_get_max_threads();
        int64_t *cnt = (int64_t *)calloc((size_t)nch + 1, sizeof(int64_t)), c;
        if (cnt) {
#pragma omp parallel for schedule(dynamic)
            for (c = 0; c < nch; c++) {
                int64_t k = 0, q;
                for (q = c * nw / nch; q < (c + 1) * nw / nch; q++) k += is_trigger(T, q, W, P);
                cnt[c + 1] = k;
            }
            for (c = 0; c < nch; c++) cnt[c + 1] += cnt[c];
#pragma omp parallel for schedule(dynamic)
            for (c = 0; c < nch; c++) {
                int64_t k = cnt[c], q;
                for (q = c * nw / nch; q < (c + 1) * nw / nch; q++)
                    if (is_trigger(T, q, W, P)) D[k++] = q + W - 1;
            }
            z = cnt[nch];
            free(cnt);
            D[z++] = n + W - 1;                          /* K:573-576 */
            return z;
        }
    }
#endif
    for (s = 0; s < nw; s++)
        if (is_trigger(T, s, W, P)) D[z++] = s + W - 1;
    D[z++] = n + W - 1;                              /* K:573-576 */
    return z;
}

/* ------------------------------------------------------------------ */
/* Generic stable merge sort with a context comparator (qsort has none). */
/* With OpenMP the two halves sort as tasks and large merges split by    */
/* divide and conquer (a pivot from the left run, its lower bound in the */
/* right run); the order is the same as the sequential stable sort.      */
/* ------------------------------------------------------------------ */
typedef int (*cmp_fn)(int64_t a, int64_t b, const void *ctx);

#define MS_PAR_MIN (1 << 15)

/* Stable merge of the sorted runs a[l1..r1) (first) and a[l2..r2) into   */
/* out[o..).  Large merges split at a pivot of the longer run: elements   */
/* of the other run that must precede it (strictly smaller when the pivot */
/* is from the first run, not larger when from the second) go left.      */
static void merge2(const int64_t *a, int64_t l1, int64_t r1, int64_t l2, int64_t r2, int64_t *out, int64_t o,
                   cmp_fn cmp, const void *ctx)
{
    const int64_t n1 = r1 - l1, n2 = r2 - l2;
    if (n1 + n2 > MS_PAR_MIN && n1 > 0 && n2 > 0) {
        int64_t i, j, lo, hi;
        if (n1 >= n2) {
            i = l1 + n1 / 2;                      /* pivot from the first run */
            lo = l2; hi = r2;
            while (lo < hi) {
                const int64_t m = lo + (hi - lo) / 2;
                if (cmp(a[m], a[i], ctx) < 0) lo = m + 1; else hi = m;
            }
            j = lo;
            out[o + (i - l1) + (j - l2)] = a[i];
#ifdef _OPENMP
#pragma omp task if ((i - l1) + (j - l2) > MS_PAR_MIN)
#endif
            merge2(a, l1, i, l2, j, out, o, cmp, ctx);
            merge2(a, i + 1, r1, j, r2, out, o + (i - l1) + (j - l2) + 1, cmp, ctx);
        } else {
            j = l2 + n2 / 2;                      /* pivot from the second run */
            lo = l1; hi = r1;
            while (lo < hi) {
                const int64_t m = lo + (hi - lo) / 2;
                if (cmp(a[j], a[m], ctx) < 0) hi = m; else lo = m + 1;
            }
            i = lo;                               /* first-run elements not larger go first */
            out[o + (i - l1) + (j - l2)] = a[j];
#ifdef _OPENMP
#pragma omp task if ((i - l1) + (j - l2) > MS_PAR_MIN)
#endif
            merge2(a, l1, i, l2, j, out, o, cmp, ctx);
            merge2(a, i, r1, j + 1, r2, out, o + (i - l1) + (j - l2) + 1, cmp, ctx);
        }
#ifdef _OPENMP
#pragma omp taskwait
#endif
        return;
    }
    {
        int64_t p = l1, q = l2, k = o;
        while (p < r1 && q < r2) out[k++] = (cmp(a[q], a[p], ctx) < 0) ? a[q++] : a[p++];
        while (p < r1) out[k++] = a[p++];
        while (q < r2) out[k++] = a[q++];
    }
}

static void msort_rec(int64_t *a, int64_t *tmp, int64_t lo, int64_t hi, cmp_fn cmp, const void *ctx)
{
    int64_t mid, i, j;
    if (hi - lo < 24) {                              /* insertion sort */
        for (i = lo + 1; i < hi; i++) {
            int64_t v = a[i];
            j = i - 1;
            while (j >= lo && cmp(a[j], v, ctx) > 0) { a[j + 1] = a[j]; j--; }
            a[j + 1] = v;
        }
        return;
    }
    mid = lo + (hi - lo) / 2;
#ifdef _OPENMP
#pragma omp task shared(a, tmp) if (hi - lo > MS_PAR_MIN)
#endif
    msort_rec(a, tmp, lo, mid, cmp, ctx);
    msort_rec(a, tmp, mid, hi, cmp, ctx);
#ifdef _OPENMP
#pragma omp taskwait
#endif
    if (cmp(a[mid - 1], a[mid], ctx) <= 0) return;
    merge2(a, lo, mid, mid, hi, tmp, lo, cmp, ctx);
    memcpy(a + lo, tmp + lo, (size_t)(hi - lo) * sizeof(int64_t));
}

static int msort(int64_t *a, int64_t n, cmp_fn cmp, const void *ctx)
{
    int64_t *tmp;
    if (n < 2) return 0;
    tmp = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    if (!tmp) return -1;
#ifdef _OPENMP
    if (n > MS_PAR_MIN) {
#pragma omp parallel
#pragma omp single
        msort_rec(a, tmp, 0, n, cmp, ctx);
    } else
#endif
        msort_rec(a, tmp, 0, n, cmp, ctx);
    free(tmp);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Phrase geometry, K:578-592 (Compute_D4): phrase k is                  */
/* X[start_k .. D[k]], start_0 = 0, start_k = D[k-1]-W+1.                */
/* ------------------------------------------------------------------ */
typedef struct {
    const uint8_t *X;   /* enlarged text, n+W bytes */
    int64_t n;
    int W;
    int64_t z;
    const int64_t *end;
    int64_t *start;
    int64_t *len;
    const int64_t *rank;     /* parse ranks for the parse-suffix comparator */
    int64_t h;
} pctx;

/* Lexicographic order of phrase occurrences; the end of a phrase is the
 * smallest symbol ("byte 0 = end", K:874, K:1008). Ties by occurrence. */
static int cmp_lex(int64_t a, int64_t b, const void *vc)
{
    const pctx *c = (const pctx *)vc;
    int64_t la = c->len[a], lb = c->len[b], m = la < lb ? la : lb;
    int r = memcmp(c->X + c->start[a], c->X + c->start[b], (size_t)m);
    if (r) return r;
    if (la != lb) return la < lb ? -1 : 1;
    return a < b ? -1 : (a > b);
}

/* Colex order of occurrences, K:1655-1677 (RadixSort_D_RL_1): characters
 * are read backwards from the phrase end; position -1 reads T[n-1], further
 * left reads 0.  Compared up to the longer length inclusive (the character
 * at distance len is the byte preceding the phrase), then by occurrence. */
static int colex_char(const pctx *c, int64_t occ, int64_t it)
{
    int64_t idx = c->end[occ] - it;
    if (idx >= 0) return c->X[idx];
    if (idx == -1) return c->X[c->n - 1];
    return 0;
}
static int cmp_colex(int64_t a, int64_t b, const void *vc)
{
    const pctx *c = (const pctx *)vc;
    int64_t m = c->len[a] > c->len[b] ? c->len[a] : c->len[b], it;
    for (it = 0; it <= m; it++) {
        int ca = colex_char(c, a, it), cb = colex_char(c, b, it);
        if (ca != cb) return ca < cb ? -1 : 1;
    }
    return a < b ? -1 : (a > b);
}

/* Parse-suffix pair comparator for prefix doubling, K:696-710: the key of
 * suffix i is (rank[i], rank[i+h]) with 0 past the end of the parse. */
static int cmp_pair(int64_t a, int64_t b, const void *vc)
{
    const pctx *c = (const pctx *)vc;
    int64_t ra = c->rank[a], rb = c->rank[b];
    if (ra != rb) return ra < rb ? -1 : 1;
    ra = a + c->h < c->z ? c->rank[a + c->h] + 1 : 0;
    rb = b + c->h < c->z ? c->rank[b + c->h] + 1 : 0;
    if (ra != rb) return ra < rb ? -1 : 1;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Stage 2-3: lexicographic sort of all occurrences + meta-characters,  */
/* K:1990-2164 (Sort_D_Left_To_Rigth), K:616-691.  The meta-character   */
/* of an occurrence is the sorted index of the last member of its group */
/* of equal phrases.  lex_rank[k] receives it; order[] the sorted order.*/
/* ------------------------------------------------------------------ */
static int lex_meta(pctx *c, int64_t *order, int64_t *meta)
{
    int64_t k, j;
    for (k = 0; k < c->z; k++) order[k] = k;
    if (msort(order, c->z, cmp_lex, c)) return GBO_NOT_ENOUGH_MEMORY;
    for (j = c->z - 1; j >= 0; j--) {
        int64_t a = order[j];
        int same_as_next = 0;
        if (j + 1 < c->z) {
            int64_t b = order[j + 1];
            same_as_next = c->len[a] == c->len[b] &&
                           memcmp(c->X + c->start[a], c->X + c->start[b], (size_t)c->len[a]) == 0;
        }
        meta[a] = same_as_next ? meta[order[j + 1]] : j;
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Stage 4: suffix array of the parse by prefix doubling, K:2342-2412.  */
/* sa[r] = start phrase of the r-th smallest parse suffix.              */
/* ------------------------------------------------------------------ */
static int parse_sa(pctx *c, const int64_t *meta, int64_t *sa)
{
    int64_t z = c->z, i, r, h;
    int64_t *rank = (int64_t *)malloc((size_t)z * sizeof(int64_t));
    int64_t *nr = (int64_t *)malloc((size_t)z * sizeof(int64_t));
    if (!rank || !nr) { free(rank); free(nr); return GBO_NOT_ENOUGH_MEMORY; }
    for (i = 0; i < z; i++) { rank[i] = meta[i]; sa[i] = i; }
    c->rank = rank;
    for (h = 1;; h <<= 1) {
        int64_t distinct = 1;
        c->h = h;
        if (msort(sa, z, cmp_pair, c)) { free(rank); free(nr); return GBO_NOT_ENOUGH_MEMORY; }
        nr[sa[0]] = 0;
        for (r = 1; r < z; r++) {
            int d = cmp_pair(sa[r - 1], sa[r], c) != 0;
            distinct += d;
            nr[sa[r]] = d ? r : nr[sa[r - 1]];
        }
        memcpy(rank, nr, (size_t)z * sizeof(int64_t));
        if (distinct == z) break;
        if (h > z) break;
    }
    free(rank); free(nr);
    return 0;
}

/* ------------------------------------------------------------------ */
/* The whole pipeline.  L receives n bytes; st (optional) the counts.   */
/* ------------------------------------------------------------------ */
typedef struct { int64_t c; int64_t len; } s_entry;  /* colex index, suffix length */

typedef struct { const pctx *p; const int64_t *colex; const s_entry *S; } sctx;

/* S entries in lexicographic order of their strings, K:4408-4552. */
static int cmp_s(int64_t a, int64_t b, const void *vc)
{
    const sctx *s = (const sctx *)vc;
    const pctx *c = s->p;
    const s_entry *ea = &s->S[a], *eb = &s->S[b];
    int64_t pa = c->end[s->colex[ea->c]] - ea->len + 1;
    int64_t pb = c->end[s->colex[eb->c]] - eb->len + 1;
    int64_t m = ea->len < eb->len ? ea->len : eb->len;
    int r = memcmp(c->X + pa, c->X + pb, (size_t)m);
    if (r) return r;
    if (ea->len != eb->len) return ea->len < eb->len ? -1 : 1;
    return a < b ? -1 : (a > b);
}

typedef struct { const int64_t *next_rank; const int64_t *colex; } mctx;
static int cmp_next(int64_t a, int64_t b, const void *vc)
{
    const mctx *m = (const mctx *)vc;
    int64_t ra = m->next_rank[m->colex[a]], rb = m->next_rank[m->colex[b]];
    if (ra != rb) return ra < rb ? -1 : 1;
    return a < b ? -1 : (a > b);
}

int gbo_pfp_bwt_ex(const uint8_t *T, int64_t n, int W, int P, int small_alphabet,
                   uint8_t *L, gbo_stats *st, int64_t *meta_out, int64_t *parse_sa_out)
{
    int rc = 0;
    int64_t z = 0, k, j, c_i, s_n = 0, max_len = 0, mixed = 0, mixed_elems = 0;
    uint8_t *X = NULL;
    int64_t *D = NULL, *start = NULL, *len = NULL, *order = NULL, *meta = NULL, *sa = NULL;
    int64_t *next_rank = NULL, *colex = NULL, *Lv = NULL, *s_idx = NULL, *blk = NULL, *dcount = NULL;
    int64_t *hi_of = NULL, *boff = NULL, max_blk = 0;
    s_entry *S = NULL;
    pctx c;

    if (W < 1 || P < 1 || n < 0 || (n > 0 && !T) || (n > 0 && !L)) return GBO_BAD_PARAMETER;
    if ((rc = gbo_validate(T, n, small_alphabet)) != 0) return rc;
    if (st) memset(st, 0, sizeof(*st));
    if (n == 0) return 0;

    X = make_enlarged(T, n, W);
    D = (int64_t *)malloc((size_t)(n + 2) * sizeof(int64_t));
    if (!X || !D) { rc = GBO_NOT_ENOUGH_MEMORY; goto done; }
    z = gbo_trigger_scan(T, n, W, P, D);

    start = (int64_t *)malloc((size_t)z * sizeof(int64_t));
    len = (int64_t *)malloc((size_t)z * sizeof(int64_t));
    order = (int64_t *)malloc((size_t)z * sizeof(int64_t));
    meta = (int64_t *)malloc((size_t)z * sizeof(int64_t));
    sa = (int64_t *)malloc((size_t)z * sizeof(int64_t));
    next_rank = (int64_t *)malloc((size_t)z * sizeof(int64_t));
    colex = (int64_t *)malloc((size_t)z * sizeof(int64_t));
    Lv = (int64_t *)malloc((size_t)z * sizeof(int64_t));
    if (!start || !len || !order || !meta || !sa || !next_rank || !colex || !Lv) { rc = GBO_NOT_ENOUGH_MEMORY; goto done; }
    for (k = 0; k < z; k++) {                        /* K:578-592 */
        start[k] = k ? D[k - 1] - W + 1 : 0;
        len[k] = D[k] - start[k] + 1;
        if (len[k] > max_len) max_len = len[k];
    }
    c.X = X; c.n = n; c.W = W; c.z = z; c.end = D; c.start = start; c.len = len; c.rank = NULL; c.h = 0;

    /* lexicographic sort + meta characters (K:1990-2164, K:616-691) */
    if ((rc = lex_meta(&c, order, meta)) != 0) goto done;
    /* parse suffix array (K:2342-2412) */
    if ((rc = parse_sa(&c, meta, sa)) != 0) goto done;
    /* rank of the next parse suffix per occurrence; last is -1 (K:787-807) */
    for (j = 0; j < z; j++) if (sa[j] >= 1) next_rank[sa[j] - 1] = j;
    next_rank[z - 1] = -1;

    /* colex sort (K:2166-2340) */
    for (k = 0; k < z; k++) colex[k] = k;
    if (msort(colex, z, cmp_colex, &c)) { rc = GBO_NOT_ENOUGH_MEMORY; goto done; }

    /* L values and S (K:2509-2592); blk[c_i] first holds the S offset of c_i */
    blk = (int64_t *)malloc((size_t)(z + 1) * sizeof(int64_t));
    if (!blk) { rc = GBO_NOT_ENOUGH_MEMORY; goto done; }
    Lv[0] = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (c_i = 1; c_i < z; c_i++) {
        int64_t a = colex[c_i], b = colex[c_i - 1], l = 0;
        while (l < len[a] && l < len[b] && X[D[a] - l] == X[D[b] - l]) l++;
        Lv[c_i] = l;
    }
    blk[0] = 0;
    for (c_i = 0; c_i < z; c_i++) {
        int64_t lo = Lv[c_i] > W ? Lv[c_i] : W;
        blk[c_i + 1] = blk[c_i] + (len[colex[c_i]] > lo ? len[colex[c_i]] - lo : 0);
    }
    s_n = blk[z];
    S = (s_entry *)malloc((size_t)(s_n ? s_n : 1) * sizeof(s_entry));
    s_idx = (int64_t *)malloc((size_t)(s_n ? s_n : 1) * sizeof(int64_t));
    if (!S || !s_idx) { rc = GBO_NOT_ENOUGH_MEMORY; goto done; }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (c_i = 0; c_i < z; c_i++) {
        int64_t lo = Lv[c_i] > W ? Lv[c_i] : W, l, t = blk[c_i];
        for (l = lo + 1; l <= len[colex[c_i]]; l++) { S[t].c = c_i; S[t].len = l; t++; }
    }
    /* lexicographic sort of S (K:4408-4552) */
    {
        sctx sc; sc.p = &c; sc.colex = colex; sc.S = S;
        for (j = 0; j < s_n; j++) s_idx[j] = j;
        if (msort(s_idx, s_n, cmp_s, &sc)) { rc = GBO_NOT_ENOUGH_MEMORY; goto done; }
    }

    /* intervals (K:2598-2764), runs (K:3247-3369), mixed blocks
     * ordered by the next parse suffix (K:3556-4248).  Every S entry's
     * interval end first (independent searches), then its block offset,
     * then the blocks in parallel. */
    hi_of = (int64_t *)malloc((size_t)(s_n ? s_n : 1) * sizeof(int64_t));
    boff = (int64_t *)malloc((size_t)(s_n + 1) * sizeof(int64_t));
    if (!hi_of || !boff) { rc = GBO_NOT_ENOUGH_MEMORY; goto done; }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1024)
#endif
    for (j = 0; j < s_n; j++) {
        const s_entry *e = &S[s_idx[j]];
        int64_t hi = e->c;
        while (hi + 1 < z && Lv[hi + 1] >= e->len) hi++;
        hi_of[j] = hi;
    }
    boff[0] = 0;
    for (j = 0; j < s_n; j++) {
        const int64_t b = hi_of[j] - S[s_idx[j]].c + 1;
        boff[j + 1] = boff[j] + b;
        if (b > max_blk) max_blk = b;
    }
    if (boff[s_n] != n) { rc = GBO_INTERNAL_ERROR; goto done; }
    {
        int failed = 0;
#ifdef _OPENMP
#pragma omp parallel reduction(+ : mixed, mixed_elems) reduction(| : failed)
#endif
        {
            int64_t *tb = (int64_t *)malloc((size_t)(max_blk ? max_blk : 1) * sizeof(int64_t)), jj;
            if (!tb) failed = 1;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
            for (jj = 0; jj < s_n; jj++) {
                const s_entry *e = &S[s_idx[jj]];
                const int64_t lo = e->c, hi = hi_of[jj], l = e->len;
                int64_t ia, ib, q, o = boff[jj];
                if (!tb) continue;
                ia = D[colex[lo]] - l; if (ia < 0) ia = n - 1;
                ib = D[colex[hi]] - l; if (ib < 0) ib = n - 1;
                if (X[ia] == X[ib]) {
                    for (q = lo; q <= hi; q++) L[o++] = X[ia];
                } else {
                    mctx mc; mc.next_rank = next_rank; mc.colex = colex;
                    for (q = lo; q <= hi; q++) tb[q - lo] = q;
                    if (msort(tb, hi - lo + 1, cmp_next, &mc)) { failed = 1; continue; }
                    for (q = 0; q <= hi - lo; q++) {
                        int64_t ip = D[colex[tb[q]]] - l;
                        if (ip < 0) ip = n - 1;
                        L[o++] = X[ip];
                    }
                    mixed++;
                    mixed_elems += hi - lo + 1;
                }
            }
            free(tb);
        }
        if (failed) { rc = GBO_NOT_ENOUGH_MEMORY; goto done; }
    }

    if (st) {
        int64_t d = 0, ld = 0;
        for (j = 0; j < z; j++) {
            int64_t a = order[j];
            if (meta[a] == j) { d++; ld += len[a]; }
        }
        st->z = z; st->d = d; st->dict_bytes = ld; st->s = s_n; st->mixed_blocks = mixed;
        st->mixed_elems = mixed_elems; st->max_phrase_len = max_len;
    }
    if (meta_out) for (k = 0; k < z; k++) meta_out[k] = meta[k];
    if (parse_sa_out) for (k = 0; k < z; k++) parse_sa_out[k] = sa[k];
    (void)dcount;

done:
    free(X); free(D); free(start); free(len); free(order); free(meta); free(sa);
    free(next_rank); free(colex); free(Lv); free(S); free(s_idx); free(blk); free(hi_of); free(boff);
    return rc;
}

int gbo_pfp_bwt(const uint8_t *T, int64_t n, int W, int P, int small_alphabet, uint8_t *L, gbo_stats *st)
{
    return gbo_pfp_bwt_ex(T, n, W, P, small_alphabet, L, st, NULL, NULL);
}

/* Number of phrases without running the whole pipeline. */
int64_t gbo_count_phrases(const uint8_t *T, int64_t n, int W, int P)
{
    int64_t z;
    int64_t *D = (int64_t *)malloc((size_t)(n + 2) * sizeof(int64_t));
    if (!D) return GBO_NOT_ENOUGH_MEMORY;
    z = gbo_trigger_scan(T, n, W, P, D);
    free(D);
    return z;
}
