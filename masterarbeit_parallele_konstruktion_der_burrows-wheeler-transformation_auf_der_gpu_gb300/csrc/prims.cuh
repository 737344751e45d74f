// prims.cuh -- device-wide scan and stable LSD radix sort (sm_103a).
//
// Scan: reduce-then-scan over tiles of 4096 items, with functor loads and
// stores so that flags, compaction and segmented heads are computed on the
// fly instead of being materialised.
//
// Radix sort: stable LSD passes over 8-bit digits.  Each pass runs a tile
// histogram (per-warp shared atomics), a digit-major exclusive scan of the
// tile histograms, and a scatter kernel that ranks keys inside each warp with
// __match_any_sync multisplit, reorders the tile in shared memory and writes
// each digit's run with consecutive addresses.  (Measured on GB300: atomics
// beat match-aggregation for counting; for the stable ranking, match beats a
// ballot-per-bit multisplit, whose ALU cost exceeds the match pipe's.)
#pragma once
#include "gbwt_internal.cuh"

namespace gbwt {

constexpr int SC_THREADS = 256;
constexpr int SC_ITEMS = 16;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

// Scan operators.  diff(inc, ex) returns a value v with op(ex, v) == inc:
// the item itself for sums, the inclusive prefix for maxima (the scan hands
// stores that v, see k_scan_down).
struct OpAdd {
    template <typename T> __device__ __forceinline__ T operator()(T a, T b) const { return a + b; }
    template <typename T> __device__ __forceinline__ T diff(T inc, T ex) const { return inc - ex; }
};
struct OpMax {
    template <typename T> __device__ __forceinline__ T operator()(T a, T b) const { return a > b ? a : b; }
    template <typename T> __device__ __forceinline__ T diff(T inc, T) const { return inc; }
};
// Component-wise max of the two 32-bit halves of a 64-bit word.
struct OpMax2 {
    __device__ __forceinline__ uint64_t operator()(uint64_t a, uint64_t b) const {
        uint32_t ah = (uint32_t)(a >> 32), bh = (uint32_t)(b >> 32);
        uint32_t al = (uint32_t)a, bl = (uint32_t)b;
        return ((uint64_t)(ah > bh ? ah : bh) << 32) | (al > bl ? al : bl);
    }
    __device__ __forceinline__ uint64_t diff(uint64_t inc, uint64_t) const { return inc; }
};
// High half: max; low half: sum (a running head with a running count).
struct OpMaxAdd {
    __device__ __forceinline__ uint64_t operator()(uint64_t a, uint64_t b) const
    {
        const uint32_t ah = (uint32_t)(a >> 32), bh = (uint32_t)(b >> 32);
        return ((uint64_t)(ah > bh ? ah : bh) << 32) | (uint32_t)((uint32_t)a + (uint32_t)b);
    }
    __device__ __forceinline__ uint64_t diff(uint64_t inc, uint64_t ex) const
    {
        return (inc & 0xFFFFFFFF00000000ull) | (uint32_t)((uint32_t)inc - (uint32_t)ex);
    }
};

// Block-wide exclusive scan (identity 0); `total` receives the block total.
template <typename T, typename Op>
__device__ __forceinline__ T block_excl_scan(T v, T &total, Op op, T *s_warp /*[32]*/)
{
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned nw = (blockDim.x + 31) >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (unsigned)o) x = op(y, x);
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? s_warp[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xFFFFFFFFu, w, o);
            if (lane >= (unsigned)o) w = op(y, w);
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    T wp = warp ? s_warp[warp - 1] : T(0);
    total = s_warp[nw - 1];
    T xe = __shfl_up_sync(0xFFFFFFFFu, x, 1);
    if (lane == 0) xe = T(0);
    __syncthreads();
    return op(wp, xe);
}

// ---- scan kernels ---------------------------------------------------
template <typename T, typename Op, typename Load>
__global__ void __launch_bounds__(SC_THREADS) k_scan_reduce(Load load, size_t n, T *partial)
{
    __shared__ T s_warp[32];
    Op op;
    size_t base = (size_t)blockIdx.x * SC_TILE;
    T acc = T(0);
#pragma unroll 4
    for (int j = 0; j < SC_ITEMS; j++) {
        size_t i = base + (size_t)j * SC_THREADS + threadIdx.x;
        if (i < n) acc = op(acc, load(i));
    }
    T total;
    block_excl_scan<T, Op>(acc, total, op, s_warp);
    if (threadIdx.x == 0) partial[blockIdx.x] = total;
}

// Stores run in striped order (consecutive threads on consecutive items, so
// a store functor's writes at i coalesce): the blocked prefixes go back
// through shared memory.  store(i, prefix, v) gets the exclusive (or
// inclusive) prefix and v = op.diff(inclusive, exclusive) -- the item's
// value for sums.
// Shared-memory slot of tile item i: one padding slot per 32 items, so the
// blocked accesses (thread t, items 16t..16t+15) hit distinct banks.
__device__ __forceinline__ uint32_t sc_pad(uint32_t i) { return i + (i >> 5); }

template <typename T, typename Op, typename Load, typename Store>
__global__ void __launch_bounds__(SC_THREADS) k_scan_down(Load load, Store store, size_t n,
                                                          const T *partial, bool inclusive,
                                                          T *total_out)
{
    __shared__ T s_tile[SC_TILE + SC_TILE / 32 + 1];
    __shared__ T s_warp[32];
    Op op;
    size_t base = (size_t)blockIdx.x * SC_TILE;
    // striped (coalesced) loads into shared memory, then blocked reads
#pragma unroll 4
    for (int j = 0; j < SC_ITEMS; j++) {
        size_t i = base + (size_t)j * SC_THREADS + threadIdx.x;
        s_tile[sc_pad(j * SC_THREADS + threadIdx.x)] = i < n ? load(i) : T(0);
    }
    __syncthreads();
    T v[SC_ITEMS];
    T sum = T(0);
#pragma unroll
    for (int j = 0; j < SC_ITEMS; j++) {
        v[j] = s_tile[sc_pad(threadIdx.x * SC_ITEMS + j)];
        sum = op(sum, v[j]);
    }
    T total;
    T ex = block_excl_scan<T, Op>(sum, total, op, s_warp);   // ends with a barrier: s_tile is free
    T run = partial ? op(partial[blockIdx.x], ex) : ex;
    // exclusive prefixes of the tile's items (items past n add the identity)
#pragma unroll
    for (int j = 0; j < SC_ITEMS; j++) {
        s_tile[sc_pad(threadIdx.x * SC_ITEMS + j)] = run;
        run = op(run, v[j]);
    }
    if (threadIdx.x == SC_THREADS - 1) s_tile[sc_pad(SC_TILE)] = run;
    __syncthreads();
#pragma unroll 4
    for (int j = 0; j < SC_ITEMS; j++) {
        const uint32_t li = (uint32_t)j * SC_THREADS + threadIdx.x;
        const size_t i = base + li;
        if (i < n) {
            const T exi = s_tile[sc_pad(li)], inc = s_tile[sc_pad(li + 1)];
            store(i, inclusive ? inc : exi, op.diff(inc, exi));
            if (total_out && i == n - 1) *total_out = inc;
        }
    }
}

template <typename T>
struct LoadArr {
    const T *a;
    __device__ __forceinline__ T operator()(size_t i) const { return a[i]; }
};
template <typename T>
struct StoreArr {
    T *a;
    __device__ __forceinline__ void operator()(size_t i, T pre, T) const { a[i] = pre; }
};

// In-place exclusive scan of a plain array (used for partials and histograms).
template <typename T, typename Op>
void scan_array_excl(Storage *st, T *a, size_t m, int depth)
{
    if (m == 0) return;
    size_t tiles = (m + SC_TILE - 1) / SC_TILE;
    if (tiles == 1) {
        k_scan_down<T, Op><<<1, SC_THREADS, 0, st->stream>>>(LoadArr<T>{a}, StoreArr<T>{a}, m,
                                                              (const T *)nullptr, false, (T *)nullptr);
        after_launch(st);
        return;
    }
    if (depth >= 3) throw Error{GBWT_INTERNAL_ERROR};
    T *part = slot<T>(st, S_SCAN1 + depth, tiles);
    k_scan_reduce<T, Op><<<(unsigned)tiles, SC_THREADS, 0, st->stream>>>(LoadArr<T>{a}, m, part);
    after_launch(st);
    scan_array_excl<T, Op>(st, part, tiles, depth + 1);
    k_scan_down<T, Op><<<(unsigned)tiles, SC_THREADS, 0, st->stream>>>(LoadArr<T>{a}, StoreArr<T>{a}, m,
                                                                        part, false, (T *)nullptr);
    after_launch(st);
}

// Scan of load(i), i in [0,n): store(i, prefix, value) is called with the
// exclusive (or inclusive) prefix.  The total is written to *total_dev when
// given (device pointer; left untouched for n == 0).
template <typename T, typename Op, typename Load, typename Store>
void device_scan(Storage *st, size_t n, Load load, Store store, bool inclusive, T *total_dev)
{
    if (n == 0) return;
    size_t tiles = (n + SC_TILE - 1) / SC_TILE;
    T *part = nullptr;
    if (tiles > 1) {
        part = slot<T>(st, S_SCAN0, tiles);
        k_scan_reduce<T, Op><<<(unsigned)tiles, SC_THREADS, 0, st->stream>>>(load, n, part);
        after_launch(st);
        scan_array_excl<T, Op>(st, part, tiles, 0);
    }
    k_scan_down<T, Op><<<(unsigned)tiles, SC_THREADS, 0, st->stream>>>(load, store, n, part, inclusive,
                                                                        total_dev);
    after_launch(st);
}

// ---------------------------------------------------------------------
// Stable LSD radix sort
// ---------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;

template <typename K>
__device__ __forceinline__ uint32_t rs_digit(K k, int shift, uint32_t mask)
{
    return (uint32_t)(k >> shift) & mask;
}

// Ranking can split its items between two warp multisplits so that both
// issue pipes work: __match_any_sync (one instruction, limited by its pipe)
// and one ballot per digit bit (ALU work); every BALLOT-th item uses ballots
// (template argument, 0 = never).  Measured on GB300 for the batched output
// sort (u32 keys, uniform 8-bit digits): 727 us per pass with match only,
// 595 us with BALLOT = 3, 580 us with BALLOT = 2.  The match instruction's
// cost grows with the number of distinct digits in a warp, so sorts whose
// warps see few distinct digits keep match only.

// Lanes of the warp holding the same digit d (< 2^BITS, or 0xFFFFFFFF for
// no key: those lanes form their own class).
template <int BITS>
__device__ __forceinline__ unsigned rs_peers_ballot(uint32_t d)
{
    const bool valid = d != 0xFFFFFFFFu;
    const unsigned vm = __ballot_sync(0xFFFFFFFFu, valid);
    unsigned m = valid ? vm : ~vm;
#pragma unroll
    for (int b = 0; b < BITS; b++) {
        const unsigned v = __ballot_sync(0xFFFFFFFFu, (d >> b) & 1u);
        m &= ((d >> b) & 1u) ? v : ~v;
    }
    return m;
}


// Histogram slot of digit d for tile b.  Unsegmented: digit-major over all
// tiles.  Segmented (tseg[b] = {first tile, tiles} of b's segment, every
// segment a whole number of tiles): segment-major, then digit-major inside
// the segment, so one exclusive scan gives every tile its offsets inside its
// own segment and each pass sorts the segments independently.
__device__ __forceinline__ size_t rs_hist_index(const uint2 *tseg, uint32_t b, uint32_t d, uint32_t num_tiles, int D)
{
    if (!tseg) return (size_t)d * num_tiles + b;
    const uint2 q = tseg[b];
    return (size_t)q.x * D + (size_t)d * q.y + (b - q.x);
}

template <typename K, int BITS>
__global__ void __launch_bounds__(RS_THREADS) k_rs_upsweep(const K *__restrict__ keys, uint32_t n, int shift,
                                                           uint32_t mask, uint32_t *__restrict__ tile_hist,
                                                           uint32_t num_tiles, const uint2 *__restrict__ tseg)
{
    constexpr int D = 1 << BITS;
    __shared__ uint32_t h[RS_WARPS * D];       // one histogram per warp
    for (int d = threadIdx.x; d < RS_WARPS * D; d += RS_THREADS) h[d] = 0;
    __syncthreads();
    uint32_t *wh = h + (threadIdx.x >> 5) * D;
    const size_t base = (size_t)blockIdx.x * RS_TILE;
    constexpr int KPV = 16 / (int)sizeof(K);          // keys per 16-byte load
    constexpr int NV = RS_ITEMS / KPV;
    if (base + RS_TILE <= n && (((uintptr_t)keys) & 15u) == 0) {
        // full tile: every load issued before any count (counting needs no order)
        uint4 v[NV];
#pragma unroll
        for (int j = 0; j < NV; j++) v[j] = __ldg((const uint4 *)(keys + base) + (size_t)j * RS_THREADS + threadIdx.x);
#pragma unroll
        for (int j = 0; j < NV; j++) {
            K kk[KPV];
            memcpy(kk, &v[j], 16);
#pragma unroll
            for (int q = 0; q < KPV; q++) atomicAdd(&wh[rs_digit(kk[q], shift, mask)], 1u);
        }
    } else {
#pragma unroll 4
        for (int j = 0; j < RS_ITEMS; j++) {
            size_t i = base + (size_t)j * RS_THREADS + threadIdx.x;
            if (i < n) atomicAdd(&wh[rs_digit(keys[i], shift, mask)], 1u);
        }
    }
    __syncthreads();
    for (int d = threadIdx.x; d < D; d += RS_THREADS) {
        uint32_t sum = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) sum += h[w * D + d];
        tile_hist[rs_hist_index(tseg, blockIdx.x, d, num_tiles, D)] = sum;
    }
}

template <typename K, bool HAS_VAL, int BITS>
constexpr size_t rs_smem_bytes()
{
    return (size_t)RS_TILE * sizeof(K) + (HAS_VAL ? (size_t)RS_TILE * 4 : 0) + (size_t)RS_WARPS * (1 << BITS) * 4 +
           (size_t)(1 << BITS) * 4 * 2 + 32 * 4;
}

template <typename K, bool HAS_VAL, int BITS, int BALLOT>
__global__ void __launch_bounds__(RS_THREADS) k_rs_downsweep(const K *__restrict__ kin, K *__restrict__ kout,
                                                             const uint32_t *__restrict__ vin,
                                                             uint32_t *__restrict__ vout, uint32_t n, int shift,
                                                             uint32_t mask, const uint32_t *__restrict__ tile_off,
                                                             uint32_t num_tiles, const uint2 *__restrict__ tseg)
{
    constexpr int D = 1 << BITS;
    constexpr int DPT = D / RS_THREADS;       // digits per thread in the per-digit phase
    extern __shared__ __align__(16) unsigned char rs_smem[];
    K *s_k = (K *)rs_smem;
    uint32_t *s_v = (uint32_t *)(s_k + RS_TILE);
    uint32_t *s_wh = HAS_VAL ? s_v + RS_TILE : s_v;
    uint32_t *s_dstart = s_wh + RS_WARPS * D;
    uint32_t *s_goff = s_dstart + D;
    uint32_t *s_scan = s_goff + D;

    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * D; i += RS_THREADS) s_wh[i] = 0;
    __syncthreads();

    const size_t tile_base = (size_t)blockIdx.x * RS_TILE;
    const size_t wbase = tile_base + (size_t)warp * (RS_ITEMS * 32);
    K k[RS_ITEMS];
    uint32_t v[RS_ITEMS];
    uint32_t rk[RS_ITEMS];
    uint32_t dg[RS_ITEMS];
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
        size_t idx = wbase + (size_t)i * 32 + lane;
        bool valid = idx < n;
        k[i] = valid ? kin[idx] : K(0);
        if (HAS_VAL) v[i] = valid ? vin[idx] : 0u;
        dg[i] = valid ? rs_digit(k[i], shift, mask) : 0xFFFFFFFFu;
    }
    uint32_t *wh = s_wh + warp * D;
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
        // the lowest lane of each digit class reads and advances the warp's
        // counter; the others take the old value from it
        const uint32_t d = dg[i];
        const unsigned peers = (BALLOT > 0 && i % (BALLOT > 0 ? BALLOT : 1) == (BALLOT > 0 ? BALLOT - 1 : 0))
                                   ? rs_peers_ballot<BITS>(d)
                                   : __match_any_sync(0xFFFFFFFFu, d);
        const unsigned leader = (unsigned)(__ffs(peers) - 1);
        uint32_t prior = 0;
        if (lane == leader && d != 0xFFFFFFFFu) {
            prior = wh[d];
            wh[d] = prior + (uint32_t)__popc(peers);
        }
        prior = __shfl_sync(0xFFFFFFFFu, prior, leader);
        rk[i] = prior + (uint32_t)__popc(peers & ((1u << lane) - 1u));
        __syncwarp();
    }
    __syncthreads();
    {
        // thread t owns digits [t*DPT, t*DPT + DPT)
        uint32_t cnt[DPT];
        uint32_t sum = 0;
#pragma unroll
        for (int e = 0; e < DPT; e++) {
            const uint32_t d = threadIdx.x * DPT + e;
            uint32_t run = 0;
#pragma unroll
            for (int w = 0; w < RS_WARPS; w++) {
                uint32_t c = s_wh[w * D + d];
                s_wh[w * D + d] = run;
                run += c;
            }
            cnt[e] = run;
            sum += run;
        }
        uint32_t total;
        uint32_t ex = block_excl_scan<uint32_t, OpAdd>(sum, total, OpAdd(), s_scan);
#pragma unroll
        for (int e = 0; e < DPT; e++) {
            const uint32_t d = threadIdx.x * DPT + e;
            s_dstart[d] = ex;
            ex += cnt[e];
            s_goff[d] = tile_off[rs_hist_index(tseg, blockIdx.x, d, num_tiles, D)];
        }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < RS_ITEMS; i++) {
        if (dg[i] != 0xFFFFFFFFu) {
            uint32_t lp = s_dstart[dg[i]] + s_wh[warp * D + dg[i]] + rk[i];
            s_k[lp] = k[i];
            if (HAS_VAL) s_v[lp] = v[i];
        }
    }
    __syncthreads();
    const uint32_t tile_n = (uint32_t)(((size_t)n - tile_base) < (size_t)RS_TILE ? ((size_t)n - tile_base) : RS_TILE);
    for (uint32_t j = threadIdx.x; j < tile_n; j += RS_THREADS) {
        K kk = s_k[j];
        uint32_t d = rs_digit(kk, shift, mask);
        size_t g = (size_t)s_goff[d] + (j - s_dstart[d]);
        kout[g] = kk;
        if (HAS_VAL) vout[g] = s_v[j];
    }
}

// Sorts (keys, vals) stably by bits [begin_bit, end_bit) with BITS-bit digits
// (8: 256 buckets; 10: 1024 buckets, fewer passes for 17..20-bit keys).  On
// return `keys` and `vals` point at the sorted data (the *_alt buffers hold
// garbage).  With `tseg` (see rs_hist_index; n a multiple of RS_TILE) every
// segment is sorted on its own.
template <typename K, bool HAS_VAL, int BITS = 8, int BALLOT = 0>
void radix_sort(Storage *st, K *&keys, K *&keys_alt, uint32_t *&vals, uint32_t *&vals_alt, uint32_t n,
                int begin_bit, int end_bit, const uint2 *tseg = nullptr)
{
    static_assert((1 << BITS) % RS_THREADS == 0, "digit count must be a multiple of the CTA size");
    if (n <= 1 || end_bit <= begin_bit) return;
    static bool attr_set = false;
    constexpr size_t smem = rs_smem_bytes<K, HAS_VAL, BITS>();
    if (!attr_set) {
        check_cuda(cudaFuncSetAttribute(k_rs_downsweep<K, HAS_VAL, BITS, BALLOT>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    const uint32_t num_tiles = (uint32_t)((n + RS_TILE - 1) / RS_TILE);
    const size_t D = (size_t)1 << BITS;
    uint32_t *hist = slot<uint32_t>(st, S_RSHIST, D * num_tiles);
    for (int shift = begin_bit; shift < end_bit; shift += BITS) {
        int bits = end_bit - shift < BITS ? end_bit - shift : BITS;
        uint32_t mask = (1u << bits) - 1u;
        k_rs_upsweep<K, BITS><<<num_tiles, RS_THREADS, 0, st->stream>>>(keys, n, shift, mask, hist, num_tiles, tseg);
        after_launch(st);
        scan_array_excl<uint32_t, OpAdd>(st, hist, D * num_tiles, 0);
        probe_begin(st, GBWT_PROBE_RADIX_SCATTER);
        k_rs_downsweep<K, HAS_VAL, BITS, BALLOT><<<num_tiles, RS_THREADS, smem, st->stream>>>(keys, keys_alt, vals, vals_alt,
                                                                                      n, shift, mask, hist, num_tiles,
                                                                                      tseg);
        probe_end(st, GBWT_PROBE_RADIX_SCATTER, (uint64_t)n * 2 * (sizeof(K) + (HAS_VAL ? 4 : 0)));
        after_launch(st);
        K *t = keys; keys = keys_alt; keys_alt = t;
        if (HAS_VAL) { uint32_t *u = vals; vals = vals_alt; vals_alt = u; }
    }
}

}  // namespace gbwt
