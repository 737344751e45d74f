/*
 * gbwt.h -- C ABI of the GB300 prefix-free-parsing (PFP) BWT library.
 *
 * The reference project is a set of stand-alone CUDA programs whose only
 * interface is `main()` reading ./input.txt and writing ./out.txt, with the
 * trigger parameters W and P fixed per binary by #define
 * (Prefix_Free_Parsing_W=5_P=16_kommentiert.cu, "K" below, K:16-23 and
 * Makefile:11-23).  Its internal API is a set of void functions over global
 * device pointers (K:36-98).  This header replaces that surface with plain
 * C entry points; the storage/return-code style follows the one real
 * library API inside the reference, libcubwt (libcubwt.cuh:32-101).
 *
 * Conventions shared by every entry point:
 *  - Return values >= 0 mean success; negative values are GBWT_* error
 *    codes.  No entry point traps or asserts on the device: where the
 *    reference asserts (K:130-132 input range, K:584-585 phrase length) this
 *    library returns an error code or handles the case.
 *  - Text bytes must lie in [2,254] (K:130-132); byte 1 is the implicit
 *    sentinel, W copies of which are appended internally (K:146-149).
 *    With GBWT_FLAG_SMALL_ALPHABET the bytes must lie in [2,15], the range
 *    in which the reference's two-symbols-per-digit packing is exact
 *    (Prefix_Free_Parsing_W=5_P=16_small_alphabet.cu:995-1002).
 *  - The output has exactly n bytes in the reference's convention
 *    (K:3325-3326, K:4776-4790): row i is the byte preceding the i-th
 *    smallest suffix of T, with T[n-1] preceding the whole text.
 *  - All device work runs on the storage's CUDA stream; calls on one
 *    storage object must not overlap.  One storage object per host thread.
 */
#ifndef GBWT_H
#define GBWT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBWT_VERSION_MAJOR 1
#define GBWT_VERSION_MINOR 0

/* Error codes; the first five keep libcubwt's values (libcubwt.cuh:32-38). */
#define GBWT_NO_ERROR              0
#define GBWT_BAD_PARAMETER        (-1)
#define GBWT_NOT_ENOUGH_MEMORY    (-2)
#define GBWT_GPU_ERROR            (-7)
#define GBWT_GPU_NOT_SUPPORTED    (-8)
#define GBWT_GPU_NOT_ENOUGH_MEMORY (-9)
#define GBWT_UNSUPPORTED_INPUT    (-5)   /* outside the variant's domain     */
#define GBWT_TIMEOUT              (-6)   /* a bounded device wait ran out    */
#define GBWT_INTERNAL_ERROR       (-10)

/* Flags. */
#define GBWT_FLAG_SMALL_ALPHABET  1u  /* the *_small_alphabet.cu variants   */
#define GBWT_FLAG_DEVICE_POINTERS 2u  /* T and L are device pointers        */
#define GBWT_FLAG_STAGE_TIMES     4u  /* record per-stage CUDA-event times  */

/* Counts of the last pipeline run on a storage object. */
typedef struct gbwt_stats {
    int64_t n;              /* text length                                   */
    int64_t z;              /* phrase occurrences (K: size_D)                */
    int64_t d;              /* distinct phrases                              */
    int64_t dict_bytes;     /* sum of distinct phrase lengths                */
    int64_t s;              /* |S|: distinct phrase suffixes longer than W   */
    int64_t s_elems;        /* (phrase, offset) pairs behind S               */
    int64_t mixed_blocks;   /* S entries whose BWT block is not one run      */
    int64_t mixed_elems;    /* BWT bytes inside mixed blocks                 */
    int64_t dict_rounds;    /* prefix-doubling rounds, dictionary sort       */
    int64_t parse_rounds;   /* prefix-doubling rounds, parse suffix array    */
    int64_t hash_retries;   /* fingerprint retries (collision or table full)  */
    int64_t kernel_launches;/* kernels launched by the last call             */
    int64_t primary_index;  /* output row of the suffix starting at T[0]
                               (libcubwt's primary index minus one)          */
    int64_t probe_launches; /* launches of the probed kernel (see below)     */
    int64_t probe_bytes;    /* their algorithmic bytes                       */
    double  probe_ms;       /* their summed CUDA-event durations             */
    float   stage_ms[8];    /* with GBWT_FLAG_STAGE_TIMES: scan, phrases,
                               dictionary, parse SA, S groups, runs, mixed,
                               total                                          */
    int64_t device_bytes;   /* device scratch held by the storage now        */
} gbwt_stats;

/*
 * Allocates a storage object (stream, scratch pools) for texts of up to
 * max_length bytes on the current CUDA device.  Replaces
 * Malloc_And_Copy_On_GPU (K:175-188) and mirrors
 * libcubwt_allocate_device_storage (libcubwt.cuh:48-57).  Scratch grows on
 * first use and is reused afterwards, so repeated calls of the same size do
 * not allocate.
 */
int64_t gbwt_allocate_device_storage(void **storage, int64_t max_length);

/* Frees a storage object (libcubwt.cuh:59). */
int64_t gbwt_free_device_storage(void *storage);

/*
 * Makes the storage issue its work on `cuda_stream` (a cudaStream_t, NULL =
 * the storage's own stream).  No counterpart in the reference, which uses
 * the default stream only; needed to time the pipeline on a caller stream.
 */
int64_t gbwt_set_stream(void *storage, void *cuda_stream);

/*
 * PFP BWT of one text: T[0..n) -> L[0..n).  Replaces the process-level
 * pipeline of the reference's main() (K:4793-4815: Compute_D K:2415-2506,
 * then Compute_S K:4330-4771) for one (W, P, small_alphabet) variant
 * (Makefile:11-23).  W in [1,64], P in [1,65535] (every entry point
 * accepts the same range; P = 1 makes every window after the first a
 * trigger, since every hash is 0 mod 1).  Returns n on success.
 */
int64_t gbwt_pfp_bwt(void *storage, const uint8_t *T, uint8_t *L, int64_t n,
                     int32_t W, int32_t P, uint32_t flags);

/*
 * PFP BWT of k independent texts in one pipeline run.  Text t is
 * T_concat[offsets[t] .. offsets[t+1]) (offsets[0] = 0, non-decreasing,
 * HOST array of k+1 entries); its BWT, exactly what gbwt_pfp_bwt returns for
 * it alone, is written to L_concat at the same offsets.  Empty texts are
 * allowed and produce nothing.  No counterpart in the reference, which
 * builds one BWT per process run (main(), K:4793-4815); a caller of the
 * reference runs the program once per text.  With GBWT_FLAG_DEVICE_POINTERS
 * T_concat and L_concat are device pointers.  Returns offsets[k].
 */
int64_t gbwt_pfp_bwt_batch(void *storage, const uint8_t *T_concat, const int64_t *offsets, int32_t k,
                           uint8_t *L_concat, int32_t W, int32_t P, uint32_t flags);

/*
 * Trigger scan only: writes the phrase end positions D[0..z) (the last is
 * n+W-1) and returns z.  Replaces Compute_D1/D2/D3 (K:443-576, driver
 * K:2415-2455).  Returns GBWT_BAD_PARAMETER when capacity < z.  Only the
 * windows starting at 1..n-W can trigger, plus the forced final trigger, so
 * z <= max(n - W + 1, 1) and capacity = n + 1 always suffices.
 */
int64_t gbwt_pfp_trigger_scan(void *storage, const uint8_t *T, int64_t n, int32_t W,
                              int32_t P, uint32_t flags, int64_t *D, int64_t capacity);

/*
 * Parse of the text: for every phrase occurrence k, the dense lexicographic
 * rank of its phrase among the distinct phrases (ranks[0..z)), and the
 * suffix array of that parse (parse_sa[0..z), may be NULL).  Replaces the
 * phrase sort + meta-characters + parse suffix array of the reference
 * (K:1990-2164, K:616-691, K:2342-2412); the reference's meta-character is
 * the sorted index of the last occurrence of an equal phrase, which orders
 * phrases exactly like the dense rank returned here.  Returns z.
 */
int64_t gbwt_pfp_parse(void *storage, const uint8_t *T, int64_t n, int32_t W, int32_t P,
                       uint32_t flags, int32_t *ranks, int32_t *parse_sa, int64_t capacity);

/*
 * Trigger scan that allocates nothing.  No counterpart in the reference: it
 * serves callers that cannot allocate device memory (a host framework that
 * hands out a fixed budget, an allocator that must not be re-entered, a
 * process that reserved all device memory up front).  T (n bytes) and D
 * (capacity uint32 slots) are DEVICE pointers owned by the caller; `stream`
 * is a cudaStream_t (NULL = legacy default stream).  Writes the phrase end
 * positions D[0..z) exactly like gbwt_pfp_trigger_scan and returns z.
 * Capacity: z <= max(n - W + 1, 1), so capacity = n + 1 always suffices;
 * a smaller capacity that turns out too small gives GBWT_BAD_PARAMETER.
 * Limits: n <= 2^30 bytes.  The scratch is one library-wide device array of
 * about 1 MiB that every GPU loading the library keeps until exit; the first
 * call on a device checks that the device is an sm_103 GPU
 * (GBWT_GPU_NOT_SUPPORTED otherwise, before any device work) and looks up
 * the array's address.  Every call reads the trigger count back between its
 * two passes and synchronises `stream` before it returns, so it must not be
 * called on a stream that is being captured into a CUDA graph.  Calls that
 * overlap on the GPU race on the shared array and must be serialised by the
 * caller; each call clears what must start at zero.
 */
int64_t gbwt_pfp_trigger_scan_noalloc(const uint8_t *T, int64_t n, int32_t W, int32_t P, uint32_t flags,
                                      uint32_t *D, int64_t capacity, void *stream);

/*
 * libcubwt-compatible BWT (libcubwt.cuh:60-69, libcubwt.cu:2414-2431):
 * L[0] = T[n-1], then the BWT of T$ without its '$' entry; returns the
 * primary index (the row where '$' stood, >= 1).  T and L are host buffers.
 * Any byte values are accepted: a text with at most 253 distinct values is
 * mapped monotonically into [2,254] (which leaves its BWT unchanged), run
 * through the PFP pipeline with W=5, P=16, and mapped back; a text using all
 * 254-256 values gives GBWT_UNSUPPORTED_INPUT.  No counterpart in the
 * reference's PFP programs; it serves callers of the vendored libcubwt.
 */
int64_t gbwt_libcubwt_bwt(void *storage, const uint8_t *T, uint8_t *L, int64_t n);

/*
 * libcubwt_bwt_aux's contract (libcubwt.cuh:80-89): the same BWT plus the
 * auxiliary indexes I[0..(n-1)/r], I[k] = row of the suffix starting at
 * k*r in libcubwt's numbering (I[0] is the primary index); r a power of two
 * >= 2.  Host pointers.  Returns GBWT_NO_ERROR.
 */
int64_t gbwt_libcubwt_bwt_aux(void *storage, const uint8_t *T, uint8_t *L, int64_t n, int64_t r, uint32_t *I);

/*
 * Inverse BWT on the GPU: L[0..n) as returned by gbwt_pfp_bwt and its
 * primary index (gbwt_stats.primary_index) -> T[0..n).  Host pointers, or
 * device pointers with GBWT_FLAG_DEVICE_POINTERS.  Returns n;
 * GBWT_BAD_PARAMETER when L is not a BWT with that primary index.  The
 * reference declares libcubwt_unbwt without defining it (libcubwt.cuh:101).
 */
int64_t gbwt_unbwt(void *storage, const uint8_t *L, uint8_t *T, int64_t n, int64_t primary, uint32_t flags);

/*
 * libcubwt_unbwt's contract (libcubwt.cuh:90-101): T is libcubwt's BWT
 * (L[0] = T[n-1], no '$' row), i its primary index, U the output (host
 * pointers; may equal T); freq may be NULL (counts are recomputed).
 * Returns GBWT_NO_ERROR.
 */
int64_t gbwt_libcubwt_unbwt(void *storage, const uint8_t *T, uint8_t *U, int64_t n, const int32_t *freq,
                            int32_t i);

/* Copies the counts of the last call into *out. */
int64_t gbwt_get_stats(void *storage, gbwt_stats *out);

/*
 * Tuning knobs of a storage object (0 = built-in default).  They change how
 * the work is scheduled, never the result.  No counterpart in the reference
 * (its launch shapes are compile-time constants); an autotuner picks them
 * per size class (package module autotune).
 */
typedef struct gbwt_tuning {
    int32_t hash_log2_max;      /* phrase hash table: at most 2^k slots (16..28; default 22)        */
    int32_t batch_seg_tiles;    /* batch: texts grouped until a sort segment holds this many
                                   4096-element tiles (1..1024; default 8)                           */
    int32_t batch_pad_eighths;  /* batch: one text per segment when tile padding is at most this
                                   many eighths of the elements (0..64; default 1)                   */
    int32_t batch_radix_bits;   /* batch output sort digit width: 8, 9, or 0 = fewest passes         */
    int32_t unbwt_rate_log2;    /* inverse BWT: one ruler per 2^k rows (2..12; default 7)            */
    int32_t dict_key_bits;      /* dictionary sort, first key: at most this many bits of recoded
                                   symbols (8..64; default 64: as many symbols as fit)             */
    int32_t parse_key_phrases;  /* parse suffix array, first round: 1 or 2 phrase ranks sorted by
                                   radix; 0 (default): one text's first round comes straight from
                                   the phrase buckets of the dictionary order, no sort (batches
                                   then sort 2 ranks)                                              */
    int32_t mixed_radix_bits;   /* mixed-block element sort digit width: 8 or 10 (default 8)       */
    int32_t batch_ballot;       /* batch output sort ranking: every k-th item by ballots (2 or 3),
                                   1 = match only (default 3)                                       */
    int32_t reserved[3];
} gbwt_tuning;

/* Sets (t != NULL) or resets (t == NULL) the storage's tuning. */
int64_t gbwt_set_tuning(void *storage, const gbwt_tuning *t);
/* Checks a tuning without a storage object: GBWT_NO_ERROR or GBWT_BAD_PARAMETER. */
int64_t gbwt_check_tuning(const gbwt_tuning *t);

/*
 * Frees the storage's scratch (it grows again on the next call).  No
 * counterpart in the reference, whose device buffers are globals freed ad
 * hoc (K:36-98); used by the serving loop to return memory to its budget.
 */
int64_t gbwt_trim_device_storage(void *storage);

/*
 * Serving loop.  No counterpart in the reference, which runs one text per
 * process (main(), K:4793-4815).  A server owns `workers` host threads, each
 * with its own storage and CUDA stream, so the work of several jobs overlaps
 * on the device.  Jobs are admitted in arrival order while the sum of the
 * running jobs' device-memory estimates stays within `hbm_budget` bytes
 * (<= 0: 80 % of the free device memory at creation); a job that does not
 * fit waits, and smaller jobs behind it may pass it.  Jobs of at most
 * `small_max` bytes (<= 0: 16 MiB) that are waiting when a worker becomes
 * free run together as one gbwt_pfp_bwt_batch call (continuous batching);
 * larger jobs run alone.  Every result is what gbwt_pfp_bwt returns for the
 * job alone.
 *
 * gbwt_submit queues T[0..n) -> L[0..n) (HOST buffers that must stay valid
 * until the job is done) and returns a ticket in *ticket; gbwt_poll and
 * gbwt_wait report the job's state in *info (may be NULL) and return
 * GBWT_JOB_PENDING, GBWT_JOB_RUNNING, GBWT_NO_ERROR (done) or the job's
 * error code.  gbwt_server_drain waits for every submitted job;
 * gbwt_server_destroy drains, then joins the workers.
 *
 * GBWT_SERVER_SIMULATE runs the scheduler without the GPU: a job "runs" for
 * n / 1 GB/s and copies T to L.  It exists to test the scheduling policy on
 * machines without a GPU.
 */
#define GBWT_SERVER_SIMULATE 0x100u
#define GBWT_JOB_PENDING 1
#define GBWT_JOB_RUNNING 2

typedef struct gbwt_job_info {
    int64_t status;         /* GBWT_JOB_*, GBWT_NO_ERROR or an error code     */
    int64_t n;              /* job length                                     */
    int64_t est_bytes;      /* device-memory estimate it was admitted with    */
    double  submit_us;      /* microseconds since the server was created      */
    double  start_us;       /* its GPU call began (0 while pending)           */
    double  end_us;         /* its result was in L (0 until done)             */
    int32_t batch_jobs;     /* jobs in the GPU call that ran it (1 = alone)   */
    int32_t worker;         /* worker that ran it                             */
} gbwt_job_info;

int64_t gbwt_server_create(void **server, int64_t hbm_budget, int32_t workers, int64_t small_max,
                           uint32_t flags);
int64_t gbwt_server_destroy(void *server);
int64_t gbwt_submit(void *server, const uint8_t *T, uint8_t *L, int64_t n, int32_t W, int32_t P,
                    uint32_t flags, int64_t *ticket);
int64_t gbwt_poll(void *server, int64_t ticket, gbwt_job_info *info);
int64_t gbwt_wait(void *server, int64_t ticket, double timeout_s, gbwt_job_info *info);
int64_t gbwt_server_drain(void *server, double timeout_s);
/* Largest sum of admitted estimates seen so far (bytes). */
int64_t gbwt_server_peak_admitted(void *server);

/* Kernels that can be probed (timed launch by launch with CUDA events). */
#define GBWT_PROBE_NONE           (-1)
#define GBWT_PROBE_RADIX_SCATTER    1   /* radix-sort scatter pass          */
#define GBWT_PROBE_TRIGGER_SCAN     2   /* trigger scan (count and write)   */
#define GBWT_PROBE_PHRASE_HASH      3   /* phrase fingerprint + table insert */
#define GBWT_PROBE_RUN_FILL         4   /* run blocks written to the output */
#define GBWT_PROBE_MIXED_SCATTER    5   /* mixed-block bytes scattered      */
#define GBWT_PROBE_SEG_SORT         6   /* prefix-doubling round, CTA groups */

/*
 * Starts timing every launch of one kernel family (GBWT_PROBE_*) on the
 * storage's stream, accumulating launches, algorithmic bytes and event time
 * into the probe_* fields of gbwt_stats across calls until the next
 * gbwt_set_kernel_probe.  No counterpart in the reference (it was profiled
 * externally with nsys, Benchmark_Skript_Linux.sh:85).
 */
int64_t gbwt_set_kernel_probe(void *storage, int32_t kernel);

/*
 * Reads the reference's input format (K:111-150, Scan_input): a decimal
 * count n, then n whitespace-separated decimal byte values.  *T is
 * malloc'ed (release with gbwt_free_host); returns n.  Values outside
 * [2,254] give GBWT_BAD_PARAMETER, where the reference asserts.
 */
int64_t gbwt_read_input_txt(const char *path, uint8_t **T, int64_t *n);

/* Writes the reference's output format (K:4776-4790, print_Output). */
int64_t gbwt_write_out_txt(const char *path, const uint8_t *L, int64_t n);

/* Releases memory returned by gbwt_read_input_txt. */
void gbwt_free_host(void *p);

/* Static description of an error code. */
const char *gbwt_error_string(int64_t code);

#ifdef __cplusplus
}
#endif

#endif /* GBWT_H */
