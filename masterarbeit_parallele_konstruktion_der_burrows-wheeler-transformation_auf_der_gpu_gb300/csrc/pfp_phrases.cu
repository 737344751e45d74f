// pfp_phrases.cu -- phrase fingerprints, exact deduplication and the
// dictionary buffer (sm_103a).
//
// The reference gives equal phrases equal ids by sorting all z occurrences
// lexicographically and pointer-jumping over equal neighbours
// (Prefix_Free_Parsing_W=5_P=16_kommentiert.cu, "K", K:1990-2164 and
// K:616-691).  Here equal phrases are found without sorting: every
// occurrence is fingerprinted (polynomial hash mod 2^61-1 over a CTA-staged
// text window), inserted into an open-addressing table sized to stay in L2
// when the dictionary is small, and then compared byte for byte with its
// table representative (the occurrence that inserted the key), so ids are
// exact.  A fingerprint collision or table overflow is detected on the
// device and the stage is re-run with a new seed or a larger table.  Which
// occurrence wins an insert varies from run to run, so internal ids may too;
// nothing downstream depends on them (phrase order comes from the
// dictionary sort), and every output is deterministic.
#include "prims.cuh"

namespace gbwt {

constexpr int PH_THREADS = 256;
constexpr int PH_SPAN = 24576;
constexpr uint64_t M61 = (1ull << 61) - 1ull;

// Phrase k spans [start, end]: end = D[k]; start = D[k-1]-W+1 (consecutive
// phrases overlap by W, K:578-592).  In a batch of texts (xsep = the padded
// buffer, see pfp_batch.cu) a phrase whose predecessor ended on a sentinel byte
// is the first phrase of the next text and starts right after it.
__device__ __forceinline__ void phrase_span(const uint32_t *D, uint32_t k, int W, const uint8_t *xsep,
                                            uint32_t &start, uint32_t &end)
{
    end = D[k];
    if (!k) { start = 0; return; }
    const uint32_t p = D[k - 1];
    start = (xsep && xsep[p] == 1) ? p + 1u : p - (uint32_t)W + 1u;
}

__device__ __forceinline__ uint64_t mulmod61(uint64_t a, uint64_t b)
{
    uint64_t lo = a * b, hi = __umul64hi(a, b);
    uint64_t r = (lo & M61) + (lo >> 61) + (hi << 3);
    r = (r & M61) + (r >> 61);
    return r >= M61 ? r - M61 : r;
}

struct HashArgs {
    const uint8_t *T;
    uint32_t n;
    const uint32_t *D;
    uint32_t z;
    int W;
    uint64_t base;          // polynomial base, < 2^61
    unsigned long long *tkeys;
    uint32_t *tvals;
    uint32_t cmask;
    int logc;
    uint32_t limit;         // distinct keys allowed before ERR_TABLE_FULL
    uint32_t *slot_of;
    uint32_t *flags;
    const uint8_t *xsep;    // batch: padded text buffer, else null
};

__global__ void __launch_bounds__(PH_THREADS) k_phrase_hash(HashArgs a)
{
    __shared__ __align__(16) uint8_t s_txt[PH_SPAN];
    const uint32_t k0 = blockIdx.x * PH_THREADS;
    const uint32_t klast = min(k0 + PH_THREADS - 1u, a.z - 1u);
    const uint32_t sa = k0 ? a.D[k0 - 1] - (uint32_t)a.W + 1u : 0u;
    const uint32_t sb = a.D[klast];
    const uint32_t a_al = sa & ~15u;
    // +32: the word reads of the last chunk may touch 12 bytes past the span
    const bool staged = (size_t)(sb - a_al) + 32 <= PH_SPAN;
    if (staged) {
        const bool aligned = (((uintptr_t)a.T) & 15u) == 0;
        const uint32_t nvec = (sb - a_al) / 16 + 1;
        for (uint32_t v = threadIdx.x; v < nvec; v += PH_THREADS) {
            uint32_t p = a_al + v * 16;
            uint4 val;
            if (aligned && (size_t)p + 16 <= a.n) {
                val = __ldg((const uint4 *)(a.T + p));
            } else {
                uint8_t b[16];
#pragma unroll
                for (int j = 0; j < 16; j++) b[j] = text_at(a.T, a.n, p + j);
                memcpy(&val, b, 16);
            }
            *(uint4 *)(s_txt + v * 16) = val;
        }
    }
    __syncthreads();
    const uint32_t k = k0 + threadIdx.x;
    if (k >= a.z) return;
    uint32_t start, end;
    phrase_span(a.D, k, a.W, a.xsep, start, end);
    const uint32_t len = end - start + 1u;
    // polynomial mod 2^61-1 over little-endian 7-byte chunks (56 bits, below
    // the modulus; the last one zero-padded)
    uint64_t h = 0;
    if (staged) {
        const uint32_t *w = (const uint32_t *)s_txt;
        for (uint32_t i = 0; i < len; i += 7) {
            const uint32_t p = start - a_al + i, q = p >> 2, sh = (p & 3u) * 8u;
            const uint32_t lo = __funnelshift_r(w[q], w[q + 1], sh), hi = __funnelshift_r(w[q + 1], w[q + 2], sh);
            uint64_t chunk = (((uint64_t)hi << 32) | lo) & 0x00FFFFFFFFFFFFFFull;
            if (len - i < 7) chunk &= (1ull << (8u * (len - i))) - 1ull;
            h = mulmod61(h, a.base) + chunk + 1u;
            if (h >= M61) h -= M61;
        }
    } else {
        for (uint32_t i = 0; i < len; i += 7) {
            uint64_t chunk = 0;
            for (uint32_t b = 0; b < 7 && i + b < len; b++)
                chunk |= (uint64_t)text_at(a.T, a.n, start + i + b) << (8 * b);
            h = mulmod61(h, a.base) + chunk + 1u;
            if (h >= M61) h -= M61;
        }
    }
    uint64_t key = h ^ ((uint64_t)len * 0x9E3779B97F4A7C15ull);
    if (key == 0) key = 1;
    uint32_t pos = (uint32_t)((key * 0xD6E8FEB86659FD93ull) >> (64 - a.logc));
    bool ok = false;
    for (uint32_t probe = 0; probe <= a.cmask; probe++) {
        // a plain read first: in a repetitive text most occurrences find
        // their key already in place, and a load costs L2 less than a CAS
        // (keys are never removed, so a key seen once stays)
        unsigned long long cur = __ldcg(a.tkeys + pos);
        if (cur == 0ull) cur = atomicCAS(a.tkeys + pos, 0ull, (unsigned long long)key);
        if (cur == 0ull) {
            // the inserting occurrence is the slot's representative
            a.tvals[pos] = k;
            uint32_t c = atomicAdd(a.flags + 1, 1u);
            if (c >= a.limit) atomicOr(a.flags, ERR_TABLE_FULL);
            ok = true;
            break;
        }
        if (cur == key) { ok = true; break; }
        pos = (pos + 1u) & a.cmask;
        if ((probe & 7u) == 7u && (*(volatile uint32_t *)a.flags & ERR_TABLE_FULL)) break;
    }
    if (!ok) {
        atomicOr(a.flags, ERR_TABLE_FULL);
        a.slot_of[k] = 0;
        return;
    }
    a.slot_of[k] = pos;
}

// 8 text bytes starting at T + p (any alignment): two aligned 8-byte loads
// and a shift.  The caller keeps T + p + 16 inside the buffer.
__device__ __forceinline__ uint64_t load8_any(const uint8_t *T, uint32_t p)
{
    const uintptr_t a = (uintptr_t)(T + p);
    const uint64_t *w = (const uint64_t *)(a & ~(uintptr_t)7);
    const uint32_t sh = (uint32_t)(a & 7u) * 8u;
    const uint64_t lo = __ldg(w), hi = __ldg(w + 1);
    return sh ? (lo >> sh) | (hi << (64u - sh)) : lo;
}

// Compares each occurrence with its representative; marks representatives.
// Inside the text 8 bytes at a time; the tail and the sentinel run after
// the text byte by byte.
__global__ void k_phrase_verify(const uint8_t *T, uint32_t n, const uint32_t *D, uint32_t z, int W,
                                const uint32_t *tvals, const uint32_t *slot_of, uint32_t *isrep, uint32_t *flags,
                                const uint8_t *xsep)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= z) return;
    const uint32_t rep = tvals[slot_of[k]];
    isrep[k] = rep == k;
    if (rep == k) return;
    if (rep >= z) { atomicOr(flags, ERR_COLLISION); return; }
    uint32_t s1, e1, s2, e2;
    phrase_span(D, k, W, xsep, s1, e1);
    phrase_span(D, rep, W, xsep, s2, e2);
    if (e1 - s1 != e2 - s2) { atomicOr(flags, ERR_COLLISION); return; }
    const uint32_t len = e1 - s1 + 1u;
    const uint32_t hi_start = s1 > s2 ? s1 : s2;
    // words only where both 16-byte load windows stay inside the n text bytes
    // (an 8-byte aligned text: the aligned loads never start before it)
    const uint32_t inside = (((uintptr_t)T & 7u) == 0 && n > hi_start + 16u) ? n - hi_start - 16u : 0u;
    const uint32_t wlen = (len < inside ? len : inside) & ~7u;
    uint32_t i = 0;
    for (; i < wlen; i += 8) {
        if (load8_any(T, s1 + i) != load8_any(T, s2 + i)) { atomicOr(flags, ERR_COLLISION); return; }
    }
    for (; i < len; i++) {
        if (text_at(T, n, s1 + i) != text_at(T, n, s2 + i)) { atomicOr(flags, ERR_COLLISION); return; }
    }
}

struct LoadU32 {
    const uint32_t *a;
    __device__ __forceinline__ uint32_t operator()(size_t i) const { return a[i]; }
};

// Dense ids in first-occurrence order: id of representative k = prefix.
struct StoreDense {
    const uint32_t *D;
    const uint32_t *slot_of;
    uint32_t *tdense;
    uint32_t *dlen;
    uint32_t *dstart;
    int W;
    const uint8_t *xsep;
    __device__ __forceinline__ void operator()(size_t k, uint32_t pre, uint32_t v) const
    {
        if (!v) return;
        uint32_t s, e;
        phrase_span(D, (uint32_t)k, W, xsep, s, e);
        tdense[slot_of[k]] = pre;
        dlen[pre] = e - s + 1u;
        dstart[pre] = s;
    }
};

// pid per occurrence; occurrence counts and the min/max preceding byte of
// every distinct phrase.
__global__ void k_phrase_finalize(const uint8_t *T, uint32_t n, const uint32_t *D, uint32_t z, int W,
                                  const uint32_t *slot_of, const uint32_t *tdense, uint32_t *pid, uint32_t *pidpc,
                                  uint32_t *occ, uint32_t *pcmin, uint32_t *pcmax, const uint8_t *xsep,
                                  const uint32_t *ptid, const uint8_t *lastb)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= z) return;
    const uint32_t id = tdense[slot_of[k]];
    pid[k] = id;
    uint32_t s, e, c;
    phrase_span(D, k, W, xsep, s, e);
    // the first phrase of a text is preceded by the text's last byte
    if (xsep && (k == 0 || xsep[D[k - 1]] == 1)) c = lastb[ptid[k]];
    else c = preceding_byte(T, n, s);
    if (pidpc) pidpc[k] = (id << 8) | c;     // only when ids fit 24 bits
    // one atomic each per occurrence: neighbouring occurrences rarely share a
    // phrase, so warp aggregation (a match per warp) costs more than it saves
    atomicAdd(occ + id, 1u);
    atomicMin(pcmin + id, c);
    atomicMax(pcmax + id, c);
}

struct LoadLen64 {
    const uint32_t *a;
    __device__ __forceinline__ uint64_t operator()(size_t i) const { return a[i]; }
};
struct StoreOff32 {
    uint32_t *a;
    __device__ __forceinline__ void operator()(size_t i, uint64_t pre, uint64_t) const { a[i] = (uint32_t)pre; }
};

// One warp per distinct phrase: copy its bytes and tag positions with the id.
__global__ void k_dict_copy(const uint8_t *T, uint32_t n, uint32_t d, const uint32_t *doff, const uint32_t *dlen,
                            const uint32_t *dstart, uint8_t *dict, uint32_t *dphr)
{
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; id < d; id += nw) {
        const uint32_t off = doff[id], len = dlen[id], st = dstart[id];
        for (uint32_t j = lane; j < len; j += 32) {
            dict[off + j] = text_at(T, n, st + j);
            dphr[off + j] = id;
        }
    }
}

static uint32_t pow2_at_least(uint64_t v)
{
    uint64_t c = 1024;
    while (c < v) c <<= 1;
    return (uint32_t)c;
}

void run_phrases(Storage *st, const uint8_t *dT, uint32_t n, int W, Phrases &ph, const BatchText *bt)
{
    const uint8_t *xsep = bt ? dT : nullptr;
    const uint32_t z = ph.z;
    uint32_t *slot_of = slot<uint32_t>(st, S_SLOT, z);
    uint32_t *isrep = slot<uint32_t>(st, S_PID, z);     // reused for pid below
    const uint32_t full_c = pow2_at_least((uint64_t)z * 2);
    const uint32_t cap = 1u << tune_hash_log2(st);       // L2-sized table while the dictionary fits
    uint32_t c = full_c < cap ? full_c : cap;
    uint64_t seed = 0x2545F4914F6CDD1Dull;
    uint32_t d = 0;
    uint32_t *tdense = nullptr, *dlen = nullptr, *dstart = nullptr;
    int attempt = 0;
    for (;; attempt++) {
        if (attempt > 6) throw Error{GBWT_INTERNAL_ERROR};
        unsigned long long *tkeys = slot<unsigned long long>(st, S_TKEYS, c);
        uint32_t *tvals = slot<uint32_t>(st, S_TVALS, c);
        tdense = slot<uint32_t>(st, S_TDENSE, c);
        dlen = slot<uint32_t>(st, S_DLEN, (size_t)z + 1);
        dstart = slot<uint32_t>(st, S_DSTART, (size_t)z + 1);
        check_cuda(cudaMemsetAsync(tkeys, 0, (size_t)c * 8, st->stream));
        check_cuda(cudaMemsetAsync(st->d_flags, 0, 8, st->stream));
        check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
        HashArgs a;
        a.T = dT; a.n = n; a.D = ph.D; a.z = z; a.W = W;
        a.base = (seed % (M61 - 1000)) + 257;
        a.tkeys = tkeys; a.tvals = tvals; a.cmask = c - 1;
        int logc = 0;
        while ((1u << logc) < c) logc++;
        a.logc = logc;
        a.limit = (uint32_t)(((uint64_t)c * 3) / 4);
        a.slot_of = slot_of; a.flags = st->d_flags; a.xsep = xsep;
        probe_begin(st, GBWT_PROBE_PHRASE_HASH);
        k_phrase_hash<<<grid_for(z, PH_THREADS), PH_THREADS, 0, st->stream>>>(a);
        // text bytes of all phrases (n + (W-1)(z-1) overlap) + D read + slot write
        probe_end(st, GBWT_PROBE_PHRASE_HASH, (uint64_t)n + (uint64_t)(W - 1) * (z - 1) + 8ull * z);
        after_launch(st);
        k_phrase_verify<<<grid_for(z, 256), 256, 0, st->stream>>>(dT, n, ph.D, z, W, tvals, slot_of, isrep,
                                                                  st->d_flags, xsep);
        after_launch(st);
        device_scan<uint32_t, OpAdd>(st, z, LoadU32{isrep}, StoreDense{ph.D, slot_of, tdense, dlen, dstart, W, xsep},
                                     false, (uint32_t *)st->d_scalars);
        check_cuda(cudaMemcpyAsync(st->h_scalars + 1, st->d_flags, 4, cudaMemcpyDeviceToHost, st->stream));
        fetch_scalars(st, 1);
        uint32_t flags = (uint32_t)(st->h_scalars[1] & 0xFFFFFFFFu);
        d = (uint32_t)(st->h_scalars[0] & 0xFFFFFFFFu);
        if (flags & ERR_TABLE_FULL) { c = full_c; st->stats.hash_retries++; continue; }
        if (flags & ERR_COLLISION) {
            seed = seed * 6364136223846793005ull + 1442695040888963407ull;
            st->stats.hash_retries++;
            continue;
        }
        break;
    }
    ph.d = d;
    uint32_t *pid = isrep;   // isrep is dead after the scan
    uint32_t *occ = slot<uint32_t>(st, S_OCC, d);
    uint32_t *pcmin = slot<uint32_t>(st, S_PCMIN, d);
    uint32_t *pcmax = slot<uint32_t>(st, S_PCMAX, d);
    check_cuda(cudaMemsetAsync(occ, 0, (size_t)d * 4, st->stream));
    check_cuda(cudaMemsetAsync(pcmin, 0xFF, (size_t)d * 4, st->stream));
    check_cuda(cudaMemsetAsync(pcmax, 0, (size_t)d * 4, st->stream));
    uint32_t *pidpc = d < (1u << 24) ? slot<uint32_t>(st, S_PIDPC, z) : nullptr;
    k_phrase_finalize<<<grid_for(z, 256), 256, 0, st->stream>>>(dT, n, ph.D, z, W, slot_of, tdense, pid, pidpc,
                                                                occ, pcmin, pcmax, xsep,
                                                                bt ? bt->ptid : nullptr,
                                                                bt ? bt->lastb : nullptr);
    ph.pidpc = pidpc;
    after_launch(st);
    // dictionary offsets (64-bit scan, checked against 2^32)
    uint32_t *doff = slot<uint32_t>(st, S_DOFF, (size_t)d + 1);
    check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
    device_scan<uint64_t, OpAdd>(st, d, LoadLen64{dlen}, StoreOff32{doff}, false, (uint64_t *)st->d_scalars);
    fetch_scalars(st, 1);
    const uint64_t dict_bytes = st->h_scalars[0];
    if (dict_bytes >= 0xFFFFFF00ull) throw Error{GBWT_UNSUPPORTED_INPUT};
    k_set_u32<<<1, 1, 0, st->stream>>>(doff + d, (uint32_t)dict_bytes);
    after_launch(st);
    uint8_t *dict = slot<uint8_t>(st, S_DICT, dict_bytes + 16);
    uint32_t *dphr = slot<uint32_t>(st, S_DPHR, dict_bytes + 1);
    unsigned blocks = grid_for((size_t)d * 32, 256);
    if (blocks > 8192) blocks = 8192;
    k_dict_copy<<<blocks, 256, 0, st->stream>>>(dT, n, d, doff, dlen, dstart, dict, dphr);
    after_launch(st);
    ph.pid = pid; ph.dlen = dlen; ph.doff = doff; ph.occ = occ; ph.pcmin = pcmin; ph.pcmax = pcmax;
    ph.dict = dict; ph.dphr = dphr; ph.dict_bytes = dict_bytes;
}

}  // namespace gbwt
