/*
 * sa_bwt.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * Independent suffix-array BWT used to pin the PFP restatement.  The suffix
 * array is built with SA-IS (induced sorting of LMS substrings), written from
 * the published method of Nong, Zhang and Chan, "Two Efficient Algorithms for
 * Linear Time Suffix Array Construction" (IEEE Trans. Computers, 2011).
 *
 * Output convention (the one the reference's PFP binaries print and that
 * compare_script.sh:7-10 checks against libcubwt): take the BWT of T$ (n+1
 * bytes), drop its first byte (the row of the suffix "$", whose byte is
 * T[n-1]) and write T[n-1] where '$' would stand.  That is libcubwt's L
 * array re-assembled at the primary index by its harness
 * (libcubwt.cu:2242-2254, libcubwt.cu:2989-3020), and the PFP output of
 * K:3325-3326 / K:3576 (preceding byte T[n-1] for the text start).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"

#define EMPTY (-1)

/* get bucket starts (end=0) or ends (end=1) */
static void buckets(const int32_t *s, int64_t n, int64_t K, int64_t *bkt, int end)
{
    int64_t i, sum = 0;
    memset(bkt, 0, (size_t)K * sizeof(int64_t));
    for (i = 0; i < n; i++) bkt[s[i]]++;
    for (i = 0; i < K; i++) {
        sum += bkt[i];
        bkt[i] = end ? sum : sum - bkt[i];
    }
}

/* s[0..n-1] over alphabet [0,K), s[n-1] == 0 unique and smallest. */
static int sais_rec(const int32_t *s, int64_t *SA, int64_t n, int64_t K)
{
    int64_t i, j, n1 = 0, name, prev;
    uint8_t *t;
    int64_t *bkt;
    int rc = 0;

    if (n == 1) { SA[0] = 0; return 0; }
    t = (uint8_t *)malloc((size_t)n);
    bkt = (int64_t *)malloc((size_t)K * sizeof(int64_t));
    if (!t || !bkt) { free(t); free(bkt); return -1; }

    /* types: 1 = S, 0 = L */
    t[n - 1] = 1;
    for (i = n - 2; i >= 0; i--)
        t[i] = (s[i] < s[i + 1] || (s[i] == s[i + 1] && t[i + 1])) ? 1 : 0;
#define ISLMS(i) ((i) > 0 && t[i] && !t[(i) - 1])

    /* step 1: place LMS positions at bucket ends and induce */
    buckets(s, n, K, bkt, 1);
    for (i = 0; i < n; i++) SA[i] = EMPTY;
    for (i = n - 1; i >= 1; i--)
        if (ISLMS(i)) SA[--bkt[s[i]]] = i;
    buckets(s, n, K, bkt, 0);
    for (i = 0; i < n; i++) {
        j = SA[i] - 1;
        if (SA[i] > 0 && !t[j]) SA[bkt[s[j]]++] = j;
    }
    buckets(s, n, K, bkt, 1);
    for (i = n - 1; i >= 0; i--) {
        j = SA[i] - 1;
        if (SA[i] > 0 && t[j]) SA[--bkt[s[j]]] = j;
    }

    /* compact sorted LMS substrings into the first n1 slots */
    for (i = 0; i < n; i++)
        if (ISLMS(SA[i])) SA[n1++] = SA[i];
    for (i = n1; i < n; i++) SA[i] = EMPTY;

    /* name LMS substrings */
    name = 0; prev = -1;
    for (i = 0; i < n1; i++) {
        int64_t pos = SA[i], d;
        int diff = 0;
        for (d = 0; d < n; d++) {
            if (prev == -1 || s[pos + d] != s[prev + d] || t[pos + d] != t[prev + d]) { diff = 1; break; }
            if (d > 0 && (ISLMS(pos + d) || ISLMS(prev + d))) break;
        }
        if (diff) { name++; prev = pos; }
        SA[n1 + pos / 2] = name - 1;
    }
    for (i = n - 1, j = n - 1; i >= n1; i--)
        if (SA[i] >= 0) SA[j--] = SA[i];

    /* step 2: sort the reduced problem */
    {
        int64_t *SA1 = SA;
        int64_t *s1l = SA + n - n1;
        if (name < n1) {
            int32_t *s1 = (int32_t *)malloc((size_t)n1 * sizeof(int32_t));
            if (!s1) { rc = -1; goto out; }
            for (i = 0; i < n1; i++) s1[i] = (int32_t)s1l[i];
            rc = sais_rec(s1, SA1, n1, name);
            free(s1);
            if (rc) goto out;
        } else {
            for (i = 0; i < n1; i++) SA1[s1l[i]] = i;
        }
        /* map reduced suffixes back to LMS positions */
        for (i = 1, j = 0; i < n; i++)
            if (ISLMS(i)) s1l[j++] = i;
        for (i = 0; i < n1; i++) SA1[i] = s1l[SA1[i]];
        for (i = n1; i < n; i++) SA[i] = EMPTY;

        /* step 3: induce the final order from sorted LMS suffixes */
        buckets(s, n, K, bkt, 1);
        for (i = n1 - 1; i >= 0; i--) {
            j = SA[i];
            SA[i] = EMPTY;
            SA[--bkt[s[j]]] = j;
        }
        buckets(s, n, K, bkt, 0);
        for (i = 0; i < n; i++) {
            j = SA[i] - 1;
            if (SA[i] > 0 && !t[j]) SA[bkt[s[j]]++] = j;
        }
        buckets(s, n, K, bkt, 1);
        for (i = n - 1; i >= 0; i--) {
            j = SA[i] - 1;
            if (SA[i] > 0 && t[j]) SA[--bkt[s[j]]] = j;
        }
    }
out:
#undef ISLMS
    free(t); free(bkt);
    return rc;
}

/* Suffix array of T (n entries, '$' row excluded). */
int gbo_suffix_array(const uint8_t *T, int64_t n, int64_t *SA)
{
    int64_t i;
    int rc;
    int32_t *s;
    int64_t *sa;
    if (n < 0) return GBO_BAD_PARAMETER;
    if (n == 0) return 0;
    s = (int32_t *)malloc((size_t)(n + 1) * sizeof(int32_t));
    sa = (int64_t *)malloc((size_t)(n + 1) * sizeof(int64_t));
    if (!s || !sa) { free(s); free(sa); return GBO_NOT_ENOUGH_MEMORY; }
    for (i = 0; i < n; i++) s[i] = (int32_t)T[i] + 1;
    s[n] = 0;
    rc = sais_rec(s, sa, n + 1, 257);
    if (!rc) memcpy(SA, sa + 1, (size_t)n * sizeof(int64_t));
    free(s); free(sa);
    return rc ? GBO_NOT_ENOUGH_MEMORY : 0;
}

int gbo_sa_bwt(const uint8_t *T, int64_t n, uint8_t *L)
{
    int64_t i;
    int rc;
    int64_t *SA;
    if (n < 0 || (n > 0 && (!T || !L))) return GBO_BAD_PARAMETER;
    if (n == 0) return 0;
    SA = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    if (!SA) return GBO_NOT_ENOUGH_MEMORY;
    rc = gbo_suffix_array(T, n, SA);
    if (!rc)
        for (i = 0; i < n; i++) L[i] = SA[i] ? T[SA[i] - 1] : T[n - 1];
    free(SA);
    return rc;
}

/* Row of the suffix starting at T[0] in the n-row output (test helper). */
int64_t gbo_primary_index(const uint8_t *T, int64_t n)
{
    int64_t i, r = -1;
    int64_t *SA;
    if (n <= 0) return -1;
    SA = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    if (!SA) return GBO_NOT_ENOUGH_MEMORY;
    if (gbo_suffix_array(T, n, SA) == 0)
        for (i = 0; i < n; i++) if (SA[i] == 0) { r = i; break; }
    free(SA);
    return r;
}

/* Inverse of the PFP-convention output: L (n bytes) with `pidx` = the row of
 * the suffix starting at T[0].  The full BWT of T$ is L' = T[n-1], L[0..n)
 * with '$' at row pidx+1; LF-mapping from the '$' row rebuilds T backwards. */
int gbo_unbwt(const uint8_t *L, int64_t n, int64_t pidx, uint8_t *T)
{
    int64_t C[257], cnt[256], i, r;
    uint32_t *LF;
    uint8_t c0;
    if (n <= 0) return 0;
    if (pidx < 0 || pidx >= n || n >= 0xFFFFFFFFll) return GBO_BAD_PARAMETER;
    c0 = L[pidx];                 /* '$' was replaced by T[n-1] */
    memset(cnt, 0, sizeof(cnt));
    for (i = 0; i < n; i++) cnt[L[i]]++;   /* L' minus '$' has the same histogram */
    C[0] = 1;
    for (i = 0; i < 256; i++) C[i + 1] = C[i] + cnt[i];
    LF = (uint32_t *)malloc((size_t)(n + 1) * sizeof(uint32_t));
    if (!LF) return GBO_NOT_ENOUGH_MEMORY;
    memset(cnt, 0, sizeof(cnt));
    for (r = 0; r <= n; r++) {
        int c;
        if (r == pidx + 1) { LF[r] = 0; continue; }
        c = r == 0 ? c0 : L[r - 1];
        LF[r] = (uint32_t)(C[c] + cnt[c]++);
    }
    r = 0;
    for (i = n - 1; i >= 0; i--) {
        T[i] = r == 0 ? c0 : L[r - 1];
        r = LF[r];
    }
    free(LF);
    return 0;
}

/* The PFP port runs its stages on one host thread. */
int gbo_threads_used(void)
{
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();      /* the PFP port's merge sorts run as OpenMP tasks */
#else
    return 1;
#endif
}

int gbo_max_threads(void)
{
#ifdef _OPENMP
    extern int omp_get_max_threads(void);
    return omp_get_max_threads();
#else
    return 1;
#endif
}
