// pfp_batch.cu -- the PFP BWT of many independent texts in one pipeline run
// (sm_103a).
//
// The reference builds one BWT per process run (main(), K:4793-4815 of
// Prefix_Free_Parsing_W=5_P=16_kommentiert.cu).  A batch of k texts runs
// the same stages once over all of them:
//
//   X      all texts in one buffer, each followed by W sentinel bytes (1);
//          input bytes are checked while copying (K:130-132).
//   scan   per-text trigger windows and forced final triggers, read from X
//          alone (pfp_scan.cu); phrase i belongs to text ptid[i].
//   dedup  one dictionary for all texts.  Within one text phrases are
//          prefix-free exactly as in its own run, so the dictionary order
//          restricted to one text's suffixes is that run's order.
//   parse  one prefix-doubling sort of every text's parse, suffixes ending
//          with their own text; restricted to one text it is that text's
//          parse suffix array.
//   output every text position becomes one element (text, dictionary group,
//          preceding byte), emitted in parse suffix order (each text's last
//          phrase first, K:787-807); a stable radix sort by (text, group)
//          leaves the elements of text t at its own output offsets, in its
//          own BWT order.  The byte payload rides in the low 8 key bits.
#include "prims.cuh"

namespace gbwt {

uint32_t run_trigger_scan_batch(Storage *st, const uint8_t *dX, uint32_t N, int W, int P, const uint32_t *xstart,
                                uint32_t k, uint32_t *&D);

constexpr int PC_THREADS = 256;
constexpr int PC_UNITS = 4;                                  // 16-byte units of X per thread
constexpr uint32_t PC_XCHUNK = PC_THREADS * PC_UNITS * 16;   // bytes of X per CTA

// Last text t < k with xstart[t] <= p, searched in [lo, hi].
__device__ __forceinline__ uint32_t text_of(const uint32_t *xstart, uint32_t lo, uint32_t hi, uint64_t p)
{
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (xstart[mid] <= p) lo = mid; else hi = mid - 1u;
    }
    return lo;
}

// X[xstart[t] + i] = Tin[ioff[t] + i]; W sentinel bytes after each text,
// zeros from N on.  Every thread writes aligned 16-byte units of X: a unit
// inside one text's bytes is four funnel shifts of five 4-byte loads
// (`words`: Tin 4-byte aligned), units at a text's end go byte by byte.
// Input bytes are checked on the way (K:130-132).
__global__ void __launch_bounds__(PC_THREADS) k_pad_copy(const uint8_t *Tin, uint64_t total, const uint32_t *ioff,
                                                         const uint32_t *xstart, uint32_t k, int W, uint32_t hi,
                                                         bool words, uint64_t N, uint8_t *X, uint32_t *flags)
{
    __shared__ uint32_t s_t0, s_t1;
    const uint64_t c0 = (uint64_t)blockIdx.x * PC_XCHUNK;
    const uint64_t c1 = c0 + PC_XCHUNK < N ? c0 + PC_XCHUNK : N;
    if (threadIdx.x == 0) {
        s_t0 = text_of(xstart, 0, k - 1u, c0);
        s_t1 = text_of(xstart, 0, k - 1u, c1 - 1u);
    }
    __syncthreads();
    const uint32_t hi4 = hi * 0x01010101u;
    uint32_t bad = 0, small_bad = 0;
#pragma unroll
    for (int u = 0; u < PC_UNITS; u++) {
        const uint64_t p = c0 + ((uint64_t)u * PC_THREADS + threadIdx.x) * 16u;
        if (p >= c1) break;
        uint32_t t = text_of(xstart, s_t0, s_t1, p);
        uint32_t xs = xstart[t];
        uint32_t len = xstart[t + 1] - xs - (uint32_t)W;
        uint32_t o[4];
        const uint64_t off = p - xs;
        const uint64_t src = (uint64_t)ioff[t] + off;
        if (words && off + 16u <= len && (src & ~3ull) + 20u <= total) {
            const uint32_t *ws = (const uint32_t *)(Tin + (src & ~3ull));
            const uint32_t sh = (uint32_t)(src & 3u) * 8u;
            uint32_t w[5];
#pragma unroll
            for (int q = 0; q < 5; q++) w[q] = __ldg(ws + q);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                o[q] = __funnelshift_r(w[q], w[q + 1], sh);
                bad |= __vcmpltu4(o[q], 0x02020202u) | __vcmpeq4(o[q], 0xFFFFFFFFu);
                small_bad |= __vcmpgtu4(o[q], hi4);
            }
        } else {
            uint8_t b[16];
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const uint64_t x = p + (uint64_t)q;
                uint32_t c = 0;
                if (x < N) {
                    while (t + 1u < k && xstart[t + 1] <= x) {
                        t++;
                        xs = xstart[t];
                        len = xstart[t + 1] - xs - (uint32_t)W;
                    }
                    const uint64_t ox = x - xs;
                    if (ox < len) {
                        c = __ldg(Tin + ioff[t] + ox);
                        bad |= (c < 2u) || (c == 255u);
                        small_bad |= c > hi;
                    } else {
                        c = 1u;
                    }
                }
                b[q] = (uint8_t)c;
            }
            memcpy(o, b, 16);
        }
        *(uint4 *)(X + p) = make_uint4(o[0], o[1], o[2], o[3]);
    }
    const bool any_bad = __any_sync(0xFFFFFFFFu, bad != 0), any_small = __any_sync(0xFFFFFFFFu, small_bad != 0);
    if ((threadIdx.x & 31u) == 0) {
        if (any_bad) atomicOr(flags, ERR_BAD_BYTE);
        else if (any_small) atomicOr(flags, ERR_SMALL_RANGE);
    }
}

__global__ void k_text_last(const uint8_t *X, const uint32_t *xstart, uint32_t k, int W, uint8_t *lastb)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < k) lastb[t] = X[xstart[t + 1] - (uint32_t)W - 1u];
}

// Text of every phrase: count of final phrases before it (a final phrase
// ends on the last sentinel byte of its text).
struct LoadFinal {
    const uint8_t *X;
    const uint32_t *D;
    __device__ __forceinline__ uint32_t operator()(size_t i) const { return X[D[i]] == 1 ? 1u : 0u; }
};
struct StoreTid {
    uint32_t *ptid;
    uint32_t *zend;
    __device__ __forceinline__ void operator()(size_t i, uint32_t pre, uint32_t v) const
    {
        ptid[i] = pre;
        if (v) zend[pre] = (uint32_t)i + 1u;
    }
};

// ---------------------------------------------------------------------
// Output elements.  Texts are grouped into segments of consecutive texts
// (a segment closes once it holds SEG_MIN elements), each padded to whole
// radix tiles.  Every text position of text t becomes one key
//   (t - first text of its segment, dictionary group, recoded byte)
// written at its segment position in text-major, parse-suffix order; one
// segmented stable radix sort then leaves each text's elements in its BWT
// order, padding (all-ones keys) at the segment ends.
// ---------------------------------------------------------------------

struct BatchLayout {
    uint32_t k = 0;                 // non-empty texts
    uint64_t total = 0, N = 0;      // text bytes; bytes of X
    uint32_t tiles = 0;             // padded element tiles
    uint32_t max_local = 1;         // most texts in one segment
    // word offsets into h_meta / the device copy
    size_t o_xstart = 0, o_ioff = 0, o_pshift = 0, o_tloc = 0, o_tseg = 0, o_tout = 0, words = 0;
};

// Text-major order of the parse suffix array: stable partition by text.
__global__ void k_text_keys(const uint32_t *psa, const uint32_t *ptid, uint32_t z, uint32_t *keys, uint32_t *vals)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= z) return;
    const uint32_t x = psa[i];
    keys[i] = ptid[x];
    vals[i] = x;
}

// Slots, text-major: text t owns slots [zs_t + t, zend_t + t] -- first its
// empty parse suffix (standing for its last phrase, K:787-807), then its
// suffixes in order (suffix x stands for phrase x-1; none when x starts the
// text).  Thread i handles the suffix at text-major position i.
struct BatchEmit {
    const uint32_t *psa, *pid, *pidpc, *D, *ptid, *zend, *dlen, *doff;
    const uint8_t *X, *lastb;
    uint32_t z;
    int W;
    const uint32_t *xstart;     // with emx: text starts in X
    uint32_t *emx;              // optional: the slot's phrase start, text-local
    __device__ __forceinline__ void fill(uint32_t occ, uint32_t s, uint32_t *emq, uint32_t *emt, uint8_t *emp,
                                         uint32_t *ecnt) const
    {
        if (emx) {
            const uint32_t t = ptid[occ];
            const bool first = occ == 0 || X[D[occ - 1]] == 1;
            emx[s] = first ? 0u : D[occ - 1] - (uint32_t)W + 1u - xstart[t];
        }
        uint32_t q, prev;
        if (pidpc) {
            const uint32_t v = pidpc[occ];
            q = v >> 8;
            prev = v & 0xFFu;
        } else {
            q = pid[occ];
            const bool first = occ == 0 || X[D[occ - 1]] == 1;
            prev = first ? lastb[ptid[occ]] : X[D[occ - 1] - (uint32_t)W];
        }
        emq[s] = doff[q];
        emt[s] = ptid[occ];
        emp[s] = (uint8_t)prev;
        ecnt[s] = dlen[q] - (uint32_t)W;
    }
};

__global__ void k_bemit_prep(BatchEmit e, uint32_t *emq, uint32_t *emt, uint8_t *emp, uint32_t *ecnt)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e.z) return;
    const uint32_t x = e.psa[i], t = e.ptid[x];
    const uint32_t zs = t ? e.zend[t - 1] : 0u;
    const uint32_t s = i + t + 1u;
    if (i == zs) e.fill(e.zend[t] - 1u, s - 1u, emq, emt, emp, ecnt);
    if (x == zs) {
        emq[s] = 0; emt[s] = t; emp[s] = 0; ecnt[s] = 0;
    } else {
        e.fill(x - 1u, s, emq, emt, emp, ecnt);
    }
}

// 256 slots per CTA; consecutive threads write consecutive elements.
constexpr int BE_T = 256;
constexpr int BE_PER = 8;
template <typename E>
__global__ void __launch_bounds__(BE_T) k_bemit(uint32_t S, const uint32_t *eoff, const uint32_t *emq,
                                                const uint32_t *emt, const uint8_t *emp, const uint32_t *pshift,
                                                const uint32_t *tloc, const uint32_t *grp_of, const uint8_t *dict,
                                                const uint8_t *enc, int gbb, int bb, E *elem, uint32_t cap,
                                                uint32_t *flags, const uint32_t *emx, uint32_t *epos)
{
    __shared__ uint32_t s_off[BE_T + 1];
    __shared__ uint32_t s_base[BE_T];
    __shared__ uint32_t s_shift[BE_T];
    __shared__ E s_hi[BE_T];
    __shared__ uint8_t s_prev[BE_T];
    __shared__ uint8_t s_enc[256];
    // staged chunk in the sc_pad layout (bank-conflict free for both orders)
    __shared__ E s_val[BE_T * BE_PER + BE_T * BE_PER / 32];
    __shared__ uint32_t s_dst[BE_T * BE_PER + BE_T * BE_PER / 32];
    __shared__ uint32_t s_pos[BE_T * BE_PER + BE_T * BE_PER / 32];
    const uint32_t t0 = blockIdx.x * BE_T;
    const uint32_t tn = min((uint32_t)BE_T, S - t0);
    s_enc[threadIdx.x] = enc[threadIdx.x];          // blockDim == 256
    if (threadIdx.x < tn) {
        const uint32_t s = t0 + threadIdx.x, t = emt[s];
        s_off[threadIdx.x] = eoff[s];
        s_base[threadIdx.x] = emq[s];
        s_shift[threadIdx.x] = pshift[t];
        s_hi[threadIdx.x] = gbb < (int)(8 * sizeof(E)) ? (E)tloc[t] << gbb : (E)0;
        s_prev[threadIdx.x] = emp[s];
    }
    if (threadIdx.x == 0) s_off[tn] = eoff[t0 + tn];
    __syncthreads();
    const uint32_t o0 = s_off[0], cnt = s_off[tn] - o0;
    // chunks of BE_T * BE_PER elements: each thread searches the slot of its
    // first element once and walks forward; the chunk is staged in shared
    // memory and written with consecutive threads on consecutive elements
    for (uint32_t cb = 0; cb < cnt; cb += BE_T * BE_PER) {
        const uint32_t e0 = cb + threadIdx.x * BE_PER;
        if (e0 < cnt) {
            uint32_t lo = 0, hi = tn - 1u;            // last slot with s_off <= o
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1u) >> 1;
                if (s_off[mid] <= o0 + e0) lo = mid; else hi = mid - 1u;
            }
#pragma unroll
            for (int q = 0; q < BE_PER; q++) {
                const uint32_t e = e0 + q;
                if (e >= cnt) break;
                const uint32_t o = o0 + e;
                while (s_off[lo + 1] <= o) lo++;
                const uint32_t j = o - s_off[lo];
                const uint32_t pos = s_base[lo] + j;
                const uint32_t c = j ? dict[pos - 1] : s_prev[lo];
                const uint32_t k = sc_pad(threadIdx.x * BE_PER + q);
                s_val[k] = s_hi[lo] | ((E)grp_of[pos] << bb) | (E)s_enc[c];
                s_dst[k] = o + s_shift[lo];
                if (epos) s_pos[k] = emx[t0 + lo] + j;     // text-local position of this suffix
            }
        }
        __syncthreads();
        const uint32_t m = min((uint32_t)(BE_T * BE_PER), cnt - cb);
        for (uint32_t i = threadIdx.x; i < m; i += BE_T) {
            const uint32_t k = sc_pad(i);
            const uint32_t dst = s_dst[k];
            if (dst < cap) {
                elem[dst] = s_val[k];
                if (epos) epos[dst] = s_pos[k];
            } else {
                atomicOr(flags, ERR_INTERNAL);
            }
        }
        __syncthreads();
    }
}

// Segment elements back to output bytes: tile b holds segment positions
// [(b - first) * RS_TILE, +RS_TILE); tout[b] = {output base, real elements}.
template <typename E>
__global__ void k_bextract(const E *elem, const uint2 *tseg, const uint2 *tout, const uint8_t *dec, uint32_t bmask,
                           uint8_t *out, const uint32_t *epos, int r_log2, uint32_t *aux)
{
    __shared__ uint8_t s_dec[256];
    s_dec[threadIdx.x] = dec[threadIdx.x];          // blockDim == 256
    __syncthreads();
    const uint32_t b = blockIdx.x;
    const uint2 sg = tseg[b], to = tout[b];
    const uint32_t p0 = (b - sg.x) * (uint32_t)RS_TILE;
    const size_t e0 = (size_t)b * RS_TILE;
    // four consecutive elements per thread: 16-byte (or 2 x 16-byte) loads
    for (uint32_t j = threadIdx.x * 4u; j < (uint32_t)RS_TILE; j += 4u * 256u) {
        const uint32_t p = p0 + j;
        if (p >= to.y) break;
        E v[4];
        if constexpr (sizeof(E) == 4) {
            const uint4 w = *(const uint4 *)(elem + e0 + j);
            memcpy(v, &w, 16);
        } else {
            const ulonglong2 w0 = *(const ulonglong2 *)(elem + e0 + j);
            const ulonglong2 w1 = *(const ulonglong2 *)(elem + e0 + j + 2);
            memcpy(v, &w0, 16);
            memcpy((char *)v + 16, &w1, 16);
        }
#pragma unroll
        for (int q = 0; q < 4; q++)
            if (p + q < to.y) out[to.x + p + q] = s_dec[(uint32_t)v[q] & bmask];
        // sampled suffix array: row (+1, libcubwt's convention) of every
        // suffix starting at a multiple of 2^r_log2 (one text per call)
        if (epos) {
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (p + q >= to.y) break;
                const uint32_t x = epos[e0 + j + q];
                if ((x & ((1u << r_log2) - 1u)) == 0) aux[x >> r_log2] = p + q + 1u;
            }
        }
    }
}

// Host layout of a batch: the non-empty texts in X, and the segments.  One
// text per segment when the tile padding costs at most pad_eighths / 8 of
// the elements (the key then needs no text bits); otherwise texts are
// grouped until a segment holds seg_tiles tiles (tuning knobs).
static BatchLayout batch_layout(Storage *st, const int64_t *offsets, int32_t k, int W)
{
    BatchLayout bl;
    bl.total = (uint64_t)offsets[k];
    uint32_t kk = 0;
    uint64_t tiles = 0, seg_real = 0, single_tiles = 0;
    for (int32_t t = 0; t < k; t++) {
        const uint64_t len = (uint64_t)(offsets[t + 1] - offsets[t]);
        if (!len) continue;
        single_tiles += (len + RS_TILE - 1) / RS_TILE;
    }
    const uint64_t pad = (uint64_t)tune_pad_eighths(st);
    const uint64_t seg_min = single_tiles * RS_TILE <= bl.total + bl.total * pad / 8
                                 ? 1u : (uint64_t)tune_seg_tiles(st) * RS_TILE;
    for (int32_t t = 0; t < k; t++) {
        const uint64_t len = (uint64_t)(offsets[t + 1] - offsets[t]);
        if (!len) continue;
        kk++;
        seg_real += len;
        if (seg_real >= seg_min) {
            tiles += (seg_real + RS_TILE - 1) / RS_TILE;
            seg_real = 0;
        }
    }
    tiles += (seg_real + RS_TILE - 1) / RS_TILE;
    if (tiles > 0xFFFFFFFFull / RS_TILE) throw Error{GBWT_UNSUPPORTED_INPUT};
    bl.k = kk;
    bl.tiles = (uint32_t)tiles;
    bl.o_xstart = 0;
    bl.o_ioff = kk + 1;
    bl.o_pshift = bl.o_ioff + kk;
    bl.o_tloc = bl.o_pshift + kk;
    bl.o_tseg = (bl.o_tloc + kk + 1) & ~(size_t)1;      // 8-byte aligned uint2 arrays
    bl.o_tout = bl.o_tseg + 2 * (size_t)bl.tiles;
    bl.words = bl.o_tout + 2 * (size_t)bl.tiles;
    if (st->h_meta_cap < bl.words) {
        if (st->h_meta) check_cuda(cudaFreeHost(st->h_meta));
        st->h_meta = nullptr;
        st->h_meta_cap = 0;
        const size_t cap = bl.words + bl.words / 4 + 1024;
        check_cuda(cudaHostAlloc(&st->h_meta, cap * sizeof(uint32_t), cudaHostAllocDefault));
        st->h_meta_cap = cap;
    }
    uint32_t *h = st->h_meta;
    uint32_t *xs = h + bl.o_xstart, *io = h + bl.o_ioff, *ps = h + bl.o_pshift, *tl = h + bl.o_tloc;
    uint32_t *tseg = h + bl.o_tseg, *tout = h + bl.o_tout;
    uint32_t i = 0, seg_first_text = 0, tile = 0;
    uint64_t x = 0, seg_obase = 0;
    seg_real = 0;
    auto close_segment = [&](uint32_t last_text) {
        const uint32_t nt = (uint32_t)((seg_real + RS_TILE - 1) / RS_TILE);
        for (uint32_t b = 0; b < nt; b++) {
            tseg[2 * (tile + b)] = tile;
            tseg[2 * (tile + b) + 1] = nt;
            tout[2 * (tile + b)] = (uint32_t)seg_obase;
            tout[2 * (tile + b) + 1] = (uint32_t)seg_real;
        }
        const uint32_t ntext = last_text - seg_first_text;
        if (ntext > bl.max_local) bl.max_local = ntext;
        // element position = output position + padding of earlier segments
        const uint32_t shift = (uint32_t)((uint64_t)tile * RS_TILE - seg_obase);
        for (uint32_t u = seg_first_text; u < last_text; u++) ps[u] = shift;
        tile += nt;
        seg_obase += seg_real;
        seg_real = 0;
        seg_first_text = last_text;
    };
    for (int32_t t = 0; t < k; t++) {
        const uint64_t len = (uint64_t)(offsets[t + 1] - offsets[t]);
        if (!len) continue;
        xs[i] = (uint32_t)x;
        io[i] = (uint32_t)offsets[t];
        tl[i] = i - seg_first_text;
        x += len + (uint64_t)W;
        seg_real += len;
        i++;
        if (seg_real >= seg_min) close_segment(i);
    }
    if (seg_real) close_segment(i);
    xs[kk] = (uint32_t)x;
    bl.N = x;
    return bl;
}

// Emission, segmented sort and extraction with E-bit keys.
template <typename E>
static void batch_output(Storage *st, const BatchLayout &bl, const uint32_t *dmeta, uint32_t S,
                         const uint32_t *eoff, const uint32_t *emq, const uint32_t *emt, const uint8_t *emp,
                         const uint32_t *grp_of, const uint8_t *dict, const uint8_t *codes, int gb, int bb, int tlb,
                         uint8_t *dOut, const uint32_t *emx, const BatchAux *aux)
{
    const uint32_t M = bl.tiles * (uint32_t)RS_TILE;
    E *elem = slot<E>(st, S_ELEM0, M);
    E *elem_alt = slot<E>(st, S_ELEM1, M);
    uint32_t *pos = aux ? slot<uint32_t>(st, S_VAL0, M) : nullptr;
    uint32_t *pos_alt = aux ? slot<uint32_t>(st, S_VAL1, M) : nullptr;
    check_cuda(cudaMemsetAsync(elem, 0xFF, (size_t)M * sizeof(E), st->stream));    // padding keys
    if (aux) check_cuda(cudaMemsetAsync(pos, 0xFF, (size_t)M * 4, st->stream));
    k_bemit<E><<<grid_for(S, BE_T), BE_T, 0, st->stream>>>(S, eoff, emq, emt, emp, dmeta + bl.o_pshift,
                                                           dmeta + bl.o_tloc, grp_of, dict, codes, gb + bb, bb, elem,
                                                           M, st->d_flags, emx, pos);
    after_launch(st);
    const uint2 *tseg = (const uint2 *)(dmeta + bl.o_tseg);
    // sort by (text, group) only: the byte rides along, and elements of one
    // group keep their parse-suffix order.  9-bit digits when they save a
    // pass (e.g. 25 group bits: 3 passes instead of 4); wider digits make the
    // 4096-key tiles' histograms (and their scan) too large.
    const int sb = tlb + gb;
    uint32_t *nv = nullptr, *nv2 = nullptr;
    const int want = st->tuning.batch_radix_bits;
    const bool nine = want ? want == 9 : (sb + 8) / 9 < (sb + 7) / 8;
    // keys-only passes rank every k-th item with ballots (uniform group
    // digits make the match-only ranking pipe-bound; tuning knob)
    const int bal = st->tuning.batch_ballot ? st->tuning.batch_ballot : 3;
    if (aux) radix_sort<E, true, 8>(st, elem, elem_alt, pos, pos_alt, M, bb, bb + sb, tseg);
    else if (nine) {
        if (bal == 2) radix_sort<E, false, 9, 2>(st, elem, elem_alt, nv, nv2, M, bb, bb + sb, tseg);
        else if (bal == 3) radix_sort<E, false, 9, 3>(st, elem, elem_alt, nv, nv2, M, bb, bb + sb, tseg);
        else radix_sort<E, false, 9, 0>(st, elem, elem_alt, nv, nv2, M, bb, bb + sb, tseg);
    } else {
        if (bal == 2) radix_sort<E, false, 8, 2>(st, elem, elem_alt, nv, nv2, M, bb, bb + sb, tseg);
        else if (bal == 3) radix_sort<E, false, 8, 3>(st, elem, elem_alt, nv, nv2, M, bb, bb + sb, tseg);
        else radix_sort<E, false, 8, 0>(st, elem, elem_alt, nv, nv2, M, bb, bb + sb, tseg);
    }
    stage_mark(st, 5);
    k_bextract<E><<<bl.tiles, 256, 0, st->stream>>>(elem, tseg, (const uint2 *)(dmeta + bl.o_tout), codes + 256,
                                                    (1u << bb) - 1u, dOut, pos, aux ? aux->r_log2 : 0,
                                                    aux ? aux->dI : nullptr);
    after_launch(st);
}

int64_t run_batch(Storage *st, const uint8_t *T, const int64_t *offsets, int32_t k, uint8_t *L, int W, int P,
                  uint32_t flags, int64_t max_n, const BatchAux *aux)
{
    if (!offsets || k < 0 || W < 1 || W > 64 || P < 1 || P > 65535) return GBWT_BAD_PARAMETER;
    if (offsets[0] != 0) return GBWT_BAD_PARAMETER;
    for (int32_t t = 0; t < k; t++)
        if (offsets[t + 1] < offsets[t]) return GBWT_BAD_PARAMETER;
    const int64_t total_i = offsets[k];
    const bool small = (flags & GBWT_FLAG_SMALL_ALPHABET) != 0;
    const bool devptr = (flags & GBWT_FLAG_DEVICE_POINTERS) != 0;
    memset(&st->stats, 0, sizeof(st->stats));
    st->launches = 0;
    st->stats.n = total_i;
    st->stage_times = (flags & GBWT_FLAG_STAGE_TIMES) != 0;
    if (total_i == 0) return 0;
    if (!T || !L) return GBWT_BAD_PARAMETER;
    // 32-bit positions inside, with room for the sentinel runs
    if ((uint64_t)total_i + (uint64_t)W * (uint64_t)k > (uint64_t)max_n) return GBWT_UNSUPPORTED_INPUT;
    const BatchLayout bl = batch_layout(st, offsets, k, W);
    const uint32_t kk = bl.k;
    const uint64_t total = bl.total, N = bl.N;

    uint32_t *meta = slot<uint32_t>(st, S_BMETA, bl.words);
    check_cuda(cudaMemcpyAsync(meta, st->h_meta, bl.words * 4, cudaMemcpyHostToDevice, st->stream));
    const uint32_t *xstart = meta + bl.o_xstart, *ioff = meta + bl.o_ioff;
    const uint8_t *dT;
    uint8_t *dOut;
    if (devptr) {
        dT = T;
        dOut = L;
    } else {
        uint8_t *buf = slot<uint8_t>(st, S_TEXT, (size_t)total + 16);
        check_cuda(cudaMemcpyAsync(buf, T, (size_t)total, cudaMemcpyHostToDevice, st->stream));
        dT = buf;
        dOut = slot<uint8_t>(st, S_OUT, (size_t)total + 16);
    }
    if (st->stage_times) check_cuda(cudaEventRecord(st->ev[0], st->stream));
    check_cuda(cudaMemsetAsync(st->d_flags, 0, 64 * sizeof(uint32_t), st->stream));
    uint8_t *X = slot<uint8_t>(st, S_BX, (size_t)N + 128);
    check_cuda(cudaMemsetAsync(X + N, 0, 128, st->stream));
    const bool words = (((uintptr_t)dT) & 3u) == 0;
    k_pad_copy<<<grid_for(N, PC_XCHUNK), PC_THREADS, 0, st->stream>>>(dT, total, ioff, xstart, kk, W,
                                                                      small ? 15u : 254u, words, N, X, st->d_flags);
    after_launch(st);
    uint8_t *lastb = slot<uint8_t>(st, S_BLAST, kk);
    k_text_last<<<grid_for(kk, 256), 256, 0, st->stream>>>(X, xstart, kk, W, lastb);
    after_launch(st);

    const uint32_t un = (uint32_t)N;
    uint32_t *D = nullptr;
    const uint32_t z = run_trigger_scan_batch(st, X, un, W, P, xstart, kk, D);
    st->stats.z = z;
    uint32_t *ptid = slot<uint32_t>(st, S_BTID, z);
    uint32_t *zend = slot<uint32_t>(st, S_BZEND, kk);
    check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
    device_scan<uint32_t, OpAdd>(st, z, LoadFinal{X, D}, StoreTid{ptid, zend}, false, (uint32_t *)st->d_scalars);
    fetch_scalars(st, 1);
    if ((uint32_t)st->h_scalars[0] != kk) throw Error{GBWT_INTERNAL_ERROR};
    stage_mark(st, 0);

    BatchText bt;
    bt.k = kk; bt.xstart = xstart; bt.ptid = ptid; bt.zend = zend; bt.lastb = lastb;
    Phrases ph;
    ph.z = z;
    ph.D = D;
    run_phrases(st, X, un, W, ph, &bt);
    st->stats.d = ph.d;
    st->stats.dict_bytes = (int64_t)ph.dict_bytes;
    stage_mark(st, 1);

    DictOrder dord;
    run_dict_sort(st, ph, W, small, dord);
    st->stats.dict_rounds = dord.rounds;
    // byte codes of the dictionary's alphabet (pinned, written by the sort):
    // code 1 is the sentinel, text bytes have codes 2.. -> output codes 0..
    uint8_t *hcodes = (uint8_t *)(st->h_scalars + 16);
    uint8_t *hpack = (uint8_t *)(st->h_scalars + 80);        // enc[256] dec[256]
    uint32_t sigma = 0;
    for (int c = 0; c < 256; c++) {
        hpack[c] = 0;
        hpack[256 + c] = 0;
    }
    for (int c = 2; c < 256; c++)
        if (hcodes[c]) {
            hpack[c] = (uint8_t)(hcodes[c] - 2);
            hpack[256 + hcodes[c] - 2] = (uint8_t)c;
            sigma++;
        }
    uint8_t *codes = slot<uint8_t>(st, S_BCODE, 512);
    check_cuda(cudaMemcpyAsync(codes, hpack, 512, cudaMemcpyHostToDevice, st->stream));
    stage_mark(st, 2);

    ParseOrder pord;
    run_parse_sa_batch(st, ph, dord, bt, pord);
    st->stats.parse_rounds = pord.rounds;
    // text-major order of the parse suffix array (stable: each text keeps its order)
    uint32_t *tkey = slot<uint32_t>(st, S_KEY0, z), *tkey2 = slot<uint32_t>(st, S_KEY1, z);
    uint32_t *tval = slot<uint32_t>(st, S_VAL0, z), *tval2 = slot<uint32_t>(st, S_VAL1, z);
    k_text_keys<<<grid_for(z, 256), 256, 0, st->stream>>>(pord.sa, ptid, z, tkey, tval);
    after_launch(st);
    radix_sort<uint32_t, true>(st, tkey, tkey2, tval, tval2, z, 0, bits_for(kk - 1u));
    const uint32_t *psa_tm = tval;
    stage_mark(st, 3);

    uint32_t *grp_of = nullptr;
    const uint32_t G = run_group_index(st, ph, dord, W, grp_of);
    if (G == 0) throw Error{GBWT_INTERNAL_ERROR};
    st->stats.s = G;
    const int tlb = bits_for(bl.max_local - 1u), gb = bits_for(G - 1u), bb = bits_for(sigma ? sigma - 1u : 0u);
    if (tlb + gb + bb > 64) throw Error{GBWT_UNSUPPORTED_INPUT};
    stage_mark(st, 4);

    const uint32_t S = kk + z;
    uint32_t *emq = slot<uint32_t>(st, S_TMP0, S);
    uint32_t *emt = slot<uint32_t>(st, S_TMP1, S);
    uint8_t *emp = slot<uint8_t>(st, S_TMP2, S);
    uint32_t *ecnt = slot<uint32_t>(st, S_GCOUNT, (size_t)S + 1);
    uint32_t *emx = aux ? slot<uint32_t>(st, S_TILEG, S) : nullptr;
    if (aux && kk != 1) throw Error{GBWT_BAD_PARAMETER};
    BatchEmit e{psa_tm, ph.pid, ph.pidpc, ph.D, ptid, zend, ph.dlen, ph.doff, X, lastb, z, W, xstart, emx};
    k_bemit_prep<<<grid_for(z, 256), 256, 0, st->stream>>>(e, emq, emt, emp, ecnt);
    after_launch(st);
    device_scan<uint32_t, OpAdd>(st, S, LoadArr<uint32_t>{ecnt}, StoreArr<uint32_t>{ecnt}, false, ecnt + S);
    check_cuda(cudaMemcpyAsync(st->d_scalars, ecnt + S, 4, cudaMemcpyDeviceToDevice, st->stream));
    fetch_scalars(st, 1);
    if ((uint32_t)st->h_scalars[0] != (uint32_t)total) throw Error{GBWT_INTERNAL_ERROR};
    st->stats.mixed_elems = (int64_t)bl.tiles * RS_TILE;     // padded element count
    if (tlb + gb + bb <= 32)
        batch_output<uint32_t>(st, bl, meta, S, ecnt, emq, emt, emp, grp_of, ph.dict, codes, gb, bb, tlb, dOut, emx,
                               aux);
    else
        batch_output<uint64_t>(st, bl, meta, S, ecnt, emq, emt, emp, grp_of, ph.dict, codes, gb, bb, tlb, dOut, emx,
                               aux);
    stage_mark(st, 6);
    if (!devptr) check_cuda(cudaMemcpyAsync(L, dOut, (size_t)total, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaMemcpyAsync(st->h_scalars + 8, st->d_flags, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                               st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    uint32_t hflags[4];
    memcpy(hflags, st->h_scalars + 8, sizeof(hflags));
    if (hflags[0] & ERR_TIMEOUT) return GBWT_TIMEOUT;
    if (hflags[0] & ERR_INTERNAL) return GBWT_INTERNAL_ERROR;
    if (st->stage_times) {
        for (int i = 0; i < 7; i++) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, st->ev[i], st->ev[i + 1]) != cudaSuccess) ms = 0.f;
            st->stats.stage_ms[i] = ms;
        }
        float tot = 0.f;
        if (cudaEventElapsedTime(&tot, st->ev[0], st->ev[7]) == cudaSuccess) st->stats.stage_ms[7] = tot;
    }
    st->stats.kernel_launches = st->launches;
    return total_i;
}

}  // namespace gbwt
