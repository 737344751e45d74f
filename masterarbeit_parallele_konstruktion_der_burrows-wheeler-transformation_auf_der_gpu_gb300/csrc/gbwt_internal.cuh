// gbwt_internal.cuh -- storage object, scratch slots, error plumbing and
// small device helpers shared by the PFP BWT kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>
#include <string.h>
#include "../../include/gbwt.h"

namespace gbwt {

// Device-side error bits, OR-ed into Storage::d_flags[0] by kernels.  No
// kernel traps; the host turns these bits into GBWT_* return codes.
enum : uint32_t {
    ERR_BAD_BYTE     = 1u << 0,   // byte outside [2,254]
    ERR_SMALL_RANGE  = 1u << 1,   // byte in [16,254] with the small-alphabet flag
    ERR_COLLISION    = 1u << 2,   // two different phrases share a fingerprint
    ERR_TABLE_FULL   = 1u << 3,   // phrase table exceeded its load limit
    ERR_INTERNAL     = 1u << 4,   // an internal consistency check failed
    ERR_TIMEOUT      = 1u << 5,   // a bounded device wait gave up
};

// Scratch slots; each grows on demand and is reused by later calls.
enum Slot : int {
    S_TEXT = 0, S_OUT,
    S_D, S_PID, S_SLOT, S_TKEYS, S_TVALS, S_TDENSE,
    S_DLEN, S_DSTART, S_DOFF, S_OCC, S_PCMIN, S_PCMAX, S_DICT, S_DPHR,
    S_KEY0, S_KEY1, S_VAL0, S_VAL1, S_ISA, S_SA, S_ACTX, S_ACTG, S_HEAD,
    S_LEXRANK, S_PARSE, S_PISA, S_PSA,
    S_GCOUNT, S_GCHAR, S_GMIX, S_GOFF, S_GRP, S_MOFF, S_MB, S_MC, S_MIXIDX, S_DELTA,
    S_ELEM0, S_ELEM1,
    S_SCAN0, S_SCAN1, S_SCAN2, S_SCAN3, S_RSHIST,
    S_TMP0, S_TMP1, S_TMP2, S_PIDPC, S_TILEG, S_ACTX2, S_ACTG2, S_LCB, S_LCBMAP,
    S_BX, S_BMETA, S_BTID, S_BZEND, S_BLAST, S_BCODE, S_SSTART,
    S_BIGL, S_BIGM,
    S_NUM
};

struct Buf { void *p = nullptr; size_t cap = 0; };

struct Storage {
    int device = 0;
    cudaStream_t stream = nullptr;      // stream in use
    cudaStream_t own_stream = nullptr;  // created by the storage
    int64_t max_length = 0;
    Buf slots[S_NUM];
    uint32_t *d_flags = nullptr;        // [0] error bits, [1..] counters
    uint64_t *h_scalars = nullptr;      // pinned host mirror (256 entries; [16..80) byte tables)
    uint64_t *d_scalars = nullptr;      // device scalars (64 entries)
    uint32_t *h_meta = nullptr;         // pinned batch layout (grows on demand)
    size_t h_meta_cap = 0;
    gbwt_tuning tuning = {};            // 0 = default for every knob
    gbwt_stats stats;
    int64_t launches = 0;
    bool stage_times = false;
    cudaEvent_t ev[10] = {};
    int num_sms = 152;
    // kernel probe: event pairs around each launch of one kernel family
    int probe_kernel = -1;
    cudaEvent_t *probe_ev = nullptr;   // 2 * probe_cap events
    int probe_cap = 0;
    int probe_used = 0;                // pairs recorded since the last harvest
    int64_t probe_launches = 0;
    int64_t probe_bytes = 0;
    double probe_ms = 0.0;
};

// Thrown inside the library and turned into return codes at the C ABI.
struct Error { int64_t code; };

inline void check_cuda(cudaError_t e)
{
    if (e == cudaSuccess) return;
    if (e == cudaErrorMemoryAllocation) throw Error{GBWT_GPU_NOT_ENOUGH_MEMORY};
    throw Error{GBWT_GPU_ERROR};
}

// Device buffer of `count` elements in slot `s` (content not preserved on growth).
template <typename T>
T *slot(Storage *st, int s, size_t count)
{
    size_t bytes = count * sizeof(T);
    if (bytes < 256) bytes = 256;
    Buf &b = st->slots[s];
    if (b.cap < bytes) {
        if (b.p) { check_cuda(cudaFree(b.p)); b.p = nullptr; b.cap = 0; }
        size_t want = bytes + bytes / 8;          // headroom for size jitter
        want = (want + 4095) & ~(size_t)4095;
        check_cuda(cudaMalloc(&b.p, want));
        b.cap = want;
    }
    return (T *)b.p;
}

// Reads `k` device scalars (d_scalars[0..k)) into host memory synchronously.
inline void fetch_scalars(Storage *st, int k)
{
    check_cuda(cudaMemcpyAsync(st->h_scalars, st->d_scalars, (size_t)k * sizeof(uint64_t),
                               cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
}

inline void after_launch(Storage *st)
{
    st->launches++;
    check_cuda(cudaGetLastError());
}

// Probe hooks around a launch of kernel family `id` (GBWT_PROBE_*).
inline void probe_begin(Storage *st, int id)
{
    if (st->probe_kernel != id) return;
    if (st->probe_used == st->probe_cap) {
        // harvest what is recorded, then reuse the pool
        check_cuda(cudaStreamSynchronize(st->stream));
        for (int i = 0; i < st->probe_used; i++) {
            float ms = 0.f;
            check_cuda(cudaEventElapsedTime(&ms, st->probe_ev[2 * i], st->probe_ev[2 * i + 1]));
            st->probe_ms += ms;
        }
        st->probe_used = 0;
    }
    check_cuda(cudaEventRecord(st->probe_ev[2 * st->probe_used], st->stream));
}
inline void probe_end(Storage *st, int id, uint64_t bytes)
{
    if (st->probe_kernel != id) return;
    check_cuda(cudaEventRecord(st->probe_ev[2 * st->probe_used + 1], st->stream));
    st->probe_used++;
    st->probe_launches++;
    st->probe_bytes += (int64_t)bytes;
}

inline unsigned grid_for(size_t n, unsigned per_block)
{
    size_t g = (n + per_block - 1) / per_block;
    return (unsigned)(g ? g : 1);
}

// Effective tuning values (defaults for 0).
inline int tune_hash_log2(const Storage *st) { return st->tuning.hash_log2_max ? st->tuning.hash_log2_max : 22; }
inline int tune_seg_tiles(const Storage *st) { return st->tuning.batch_seg_tiles ? st->tuning.batch_seg_tiles : 8; }
inline int tune_pad_eighths(const Storage *st) { return st->tuning.batch_pad_eighths ? st->tuning.batch_pad_eighths : 1; }
inline int tune_unbwt_rate_log2(const Storage *st) { return st->tuning.unbwt_rate_log2 ? st->tuning.unbwt_rate_log2 : 7; }
inline int tune_dict_key_bits(const Storage *st) { return st->tuning.dict_key_bits ? st->tuning.dict_key_bits : 64; }
// 0 (default): single-text parse round 0 from the phrase buckets, no sort
// (the batch parse then sorts two phrase ranks); 1 or 2: a radix sort of
// the first one or two phrase ranks.
inline int tune_parse_key_phrases(const Storage *st) { return st->tuning.parse_key_phrases; }

inline int bits_for(uint64_t v)   // bits needed to represent values in [0, v]
{
    int b = 0;
    while (b < 64 && (v >> b)) b++;
    return b;
}

// ---------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << lane_id()) - 1u; }

// Text byte with the reference's implicit sentinel: positions n..n+W-1
// read byte 1 (K:146-149).
__device__ __forceinline__ uint8_t text_at(const uint8_t *T, uint32_t n, uint32_t i)
{
    return i < n ? __ldg(T + i) : (uint8_t)1;
}

// Byte preceding text position p in the reference's cyclic convention:
// position 0 is preceded by T[n-1] (K:1670-1677, K:3325-3326).
__device__ __forceinline__ uint8_t preceding_byte(const uint8_t *T, uint32_t n, uint32_t p)
{
    return p ? __ldg(T + p - 1) : __ldg(T + n - 1);
}

// Writes one value (kept per translation unit).
static __global__ void k_set_u32(uint32_t *p, uint32_t v) { *p = v; }

// Host-side declarations of the pipeline stages (implemented in the .cu files).
uint32_t run_trigger_scan(Storage *st, const uint8_t *dT, uint32_t n, int W, int P, bool small,
                          uint32_t *&D);
struct Phrases {
    uint32_t z = 0, d = 0;
    uint64_t dict_bytes = 0;
    const uint32_t *D = nullptr;       // [z] phrase end positions
    uint32_t *pid = nullptr;           // [z] distinct id per occurrence
    uint32_t *pidpc = nullptr;         // [z] id << 8 | preceding byte (d < 2^24), else null
    uint32_t *dlen = nullptr;          // [d] length of distinct phrase
    uint32_t *doff = nullptr;          // [d+1] offset in dictionary buffer
    uint32_t *occ = nullptr;           // [d] occurrences
    uint32_t *pcmin = nullptr, *pcmax = nullptr;  // [d] min/max preceding byte
    uint8_t *dict = nullptr;           // [dict_bytes] concatenated phrases
    uint32_t *dphr = nullptr;          // [dict_bytes] phrase id per position
};
// A batch of texts laid out in one padded buffer X: text t at xstart[t],
// followed by W sentinel bytes (value 1) that no text byte can take.  A
// phrase whose predecessor ends on a sentinel starts the next text.
struct BatchText {
    uint32_t k = 0;                    // texts (all non-empty)
    const uint32_t *xstart = nullptr;  // [k+1] text starts in X (xstart[k] = N)
    const uint32_t *ptid = nullptr;    // [z] text of each phrase
    const uint32_t *zend = nullptr;    // [k] one past the last phrase of each text
    const uint8_t *lastb = nullptr;    // [k] last byte of each text
};
void run_phrases(Storage *st, const uint8_t *dT, uint32_t n, int W, Phrases &ph, const BatchText *bt = nullptr);

struct DictOrder {
    uint32_t *isa = nullptr;     // [dict_bytes] final group head per position
    uint32_t *sa = nullptr;      // [dict_bytes] positions in sorted order
    uint32_t *lexrank = nullptr; // [d] dense lexicographic rank of each phrase
    int rounds = 0;
};
void run_dict_sort(Storage *st, Phrases &ph, int W, bool small, DictOrder &dord);

struct ParseOrder {
    uint32_t *sa = nullptr;      // [z] suffix array of the parse
    uint32_t *isa = nullptr;     // [z] inverse
    int rounds = 0;
};
void run_parse_sa(Storage *st, Phrases &ph, DictOrder &dord, ParseOrder &pord);
void run_parse_sa_batch(Storage *st, Phrases &ph, DictOrder &dord, const BatchText &bt, ParseOrder &pord);
// Group index of every dictionary position that starts a suffix longer than
// W (equal suffixes share one group; groups numbered in dictionary order).
uint32_t run_group_index(Storage *st, Phrases &ph, DictOrder &dord, int W, uint32_t *&grp_of);

void run_assembly(Storage *st, const uint8_t *dT, uint32_t n, int W, Phrases &ph,
                  DictOrder &dord, ParseOrder &pord, uint8_t *dOut);

void stage_mark(Storage *st, int idx);

void pfp_to_libcubwt(Storage *st, const uint8_t *dO, uint32_t n, uint32_t p, uint8_t *dLc);
void run_unbwt(Storage *st, const uint8_t *dLc, uint32_t n, uint32_t i, uint8_t *dT);

// Sampled suffix array of a one-text batch: aux[p >> r_log2] = row + 1 of
// the suffix starting at p, for every p that is a multiple of 2^r_log2.
struct BatchAux {
    int r_log2 = 0;
    uint32_t *dI = nullptr;     // device, (n-1) / 2^r_log2 + 1 entries
};
int64_t run_batch(Storage *st, const uint8_t *T, const int64_t *offsets, int32_t k, uint8_t *L, int W, int P,
                  uint32_t flags, int64_t max_n, const BatchAux *aux = nullptr);

}  // namespace gbwt
