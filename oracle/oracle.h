/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY (the oracle).
 * CPU restatement of the reference's PFP BWT and an independent suffix-array
 * BWT.  Loaded by tests/, __graft_entry__.smoke() and the CPU legs of
 * bench.py; never by the product path.
 */
#ifndef GBWT_ORACLE_H
#define GBWT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes share their values with include/gbwt.h. */
#define GBO_BAD_PARAMETER      (-1)
#define GBO_NOT_ENOUGH_MEMORY  (-2)
#define GBO_UNSUPPORTED_INPUT  (-5)
#define GBO_INTERNAL_ERROR     (-10)

typedef struct {
    int64_t z;              /* phrase occurrences (size_D)                */
    int64_t d;              /* distinct phrases                           */
    int64_t dict_bytes;     /* sum of distinct phrase lengths             */
    int64_t s;              /* |S|: distinct phrase suffixes longer than W */
    int64_t mixed_blocks;   /* S entries whose block is not a single run   */
    int64_t mixed_elems;    /* BWT bytes inside mixed blocks               */
    int64_t max_phrase_len;
} gbo_stats;

int     gbo_validate(const uint8_t *T, int64_t n, int small_alphabet);
int64_t gbo_trigger_scan(const uint8_t *T, int64_t n, int W, int P, int64_t *D);
int64_t gbo_count_phrases(const uint8_t *T, int64_t n, int W, int P);
int     gbo_pfp_bwt(const uint8_t *T, int64_t n, int W, int P, int small_alphabet,
                    uint8_t *L, gbo_stats *st);
int     gbo_pfp_bwt_ex(const uint8_t *T, int64_t n, int W, int P, int small_alphabet,
                       uint8_t *L, gbo_stats *st, int64_t *meta_out, int64_t *parse_sa_out);

/* Suffix-array BWT (SA-IS), output in the PFP convention: n bytes. */
int     gbo_sa_bwt(const uint8_t *T, int64_t n, uint8_t *L);
/* Plain suffix array of T (n entries) for tests. */
int     gbo_suffix_array(const uint8_t *T, int64_t n, int64_t *SA);
/* Output row of the suffix starting at T[0]; inverse BWT of the output. */
int64_t gbo_primary_index(const uint8_t *T, int64_t n);
int     gbo_unbwt(const uint8_t *L, int64_t n, int64_t pidx, uint8_t *T);

/* Threads used by the parallel parts (OpenMP); 1 when built without it. */
int     gbo_max_threads(void);
int     gbo_threads_used(void);

#ifdef __cplusplus
}
#endif
#endif
