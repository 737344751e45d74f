// pfp_unbwt.cu -- inverse BWT on the GPU (sm_103a).
//
// The reference declares libcubwt_unbwt but does not define it
// (libcubwt.cuh:101; its LF kernels are at libcubwt.cu:2453-2925).  Here:
//
//   B      the full BWT of T$ (n+1 rows, '$' at row i = libcubwt's primary
//          index); the n non-'$' rows are libcubwt's L.
//   LF     LF(r) = 1 + (position of row r in the stable sort of the non-'$'
//          rows by symbol), LF($ row) = 0.  One counting pass: tile
//          histograms, a digit-major scan, and a ranking pass (warp match
//          multisplit, as in the radix downsweep) that writes LF in row
//          order, so nothing is scattered.
//   walk   T[n-1-k] = B[LF^k(0)].  Rows whose hash falls in 1/rate are
//          rulers (row 0 always); an LF entry whose target is a ruler holds
//          bit 31 | the ruler's index.  One thread per ruler follows LF to
//          the next ruler and records the distance; pointer jumping over
//          the ruler chain gives every ruler its distance from row 0; a
//          second walk writes every text byte.  The symbol of a row comes
//          from the bucket its LF value falls in, so a step reads one word.
// Walks end at the next ruler; the rulers split the single LF cycle, so the
// steps of all walks sum to n+1.  A BWT whose LF has more than one cycle is
// rejected (the ruler chain from row 0 is not one list through all rulers,
// or does not come back to row 0 after n+1 steps).
#include "prims.cuh"

namespace gbwt {

constexpr uint32_t UB_RULER = 0x80000000u;
constexpr uint32_t UB_NIL = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t ub_mix(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x85EBCA6Bu;
    x ^= x >> 13;
    x *= 0xC2B2AE35u;
    x ^= x >> 16;
    return x;
}
__device__ __forceinline__ bool ub_is_ruler(uint32_t r, uint32_t rate_mask)
{
    return r == 0 || (ub_mix(r) & rate_mask) == 0;
}

// libcubwt's L from the PFP output O and its primary row p: O[p], O[0..p), O[p+1..n).
__global__ void k_pfp_to_libcubwt(const uint8_t *O, uint32_t n, uint32_t p, uint8_t *Lc)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    Lc[e] = e == 0 ? O[p] : (e <= p ? O[e - 1] : O[e]);
}

// Index of ruler row t in the sorted ruler list.
__device__ __forceinline__ uint32_t ub_ruler_index(const uint32_t *rul, uint32_t m, uint32_t t)
{
    uint32_t lo = 0, hi = m - 1u;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (rul[mid] < t) lo = mid + 1u; else hi = mid;
    }
    return lo;
}

// LF of every row.  Element e of Lc is row e (e < i) or e+1 (e >= i).  An
// entry whose target row is a ruler holds UB_RULER | the ruler's index.
template <int BITS>
__global__ void __launch_bounds__(RS_THREADS) k_lf_rank(const uint8_t *__restrict__ Lc, uint32_t n, uint32_t i,
                                                        const uint32_t *__restrict__ tile_off, uint32_t num_tiles,
                                                        uint32_t rate_mask, const uint32_t *__restrict__ rul,
                                                        uint32_t m, uint32_t *__restrict__ LF)
{
    constexpr int D = 1 << BITS;
    constexpr int DPT = D / RS_THREADS;
    __shared__ uint32_t s_wh[RS_WARPS * D];
    __shared__ uint32_t s_goff[D];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int q = threadIdx.x; q < RS_WARPS * D; q += RS_THREADS) s_wh[q] = 0;
    __syncthreads();
    const size_t tile_base = (size_t)blockIdx.x * RS_TILE;
    const size_t wbase = tile_base + (size_t)warp * (RS_ITEMS * 32);
    uint32_t dg[RS_ITEMS], rk[RS_ITEMS];
    uint32_t *wh = s_wh + warp * D;
#pragma unroll
    for (int q = 0; q < RS_ITEMS; q++) {
        const size_t idx = wbase + (size_t)q * 32 + lane;
        dg[q] = idx < n ? (uint32_t)Lc[idx] : 0xFFFFFFFFu;
    }
#pragma unroll
    for (int q = 0; q < RS_ITEMS; q++) {
        // the lowest lane of each digit class reads and advances the warp's
        // counter; the others take the old value from it
        const uint32_t d = dg[q];
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const unsigned leader = (unsigned)(__ffs(peers) - 1);
        uint32_t prior = 0;
        if (lane == leader && d != 0xFFFFFFFFu) {
            prior = wh[d];
            wh[d] = prior + (uint32_t)__popc(peers);
        }
        prior = __shfl_sync(0xFFFFFFFFu, prior, leader);
        rk[q] = prior + (uint32_t)__popc(peers & ((1u << lane) - 1u));
        __syncwarp();
    }
    __syncthreads();
    // per digit: exclusive prefix over the warps, and the tile's global offset
#pragma unroll
    for (int e = 0; e < DPT; e++) {
        const uint32_t d = threadIdx.x * DPT + e;
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) {
            const uint32_t c = s_wh[w * D + d];
            s_wh[w * D + d] = run;
            run += c;
        }
        s_goff[d] = tile_off[(size_t)d * num_tiles + blockIdx.x];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < RS_ITEMS; q++) {
        const uint32_t d = dg[q];
        if (d == 0xFFFFFFFFu) continue;
        const size_t e = wbase + (size_t)q * 32 + lane;
        // position among all non-'$' rows of this symbol's bucket
        const uint32_t t = 1u + s_goff[d] + s_wh[warp * D + d] + rk[q];
        const uint32_t row = (uint32_t)e < i ? (uint32_t)e : (uint32_t)e + 1u;
        LF[row] = ub_is_ruler(t, rate_mask) ? (UB_RULER | ub_ruler_index(rul, m, t)) : t;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) LF[i] = UB_RULER | 0u;      // '$' row -> row 0 = ruler 0
}

struct LoadRuler {
    uint32_t rate_mask;
    __device__ __forceinline__ uint32_t operator()(size_t r) const
    {
        return ub_is_ruler((uint32_t)r, rate_mask) ? 1u : 0u;
    }
};
struct StoreRuler {
    uint32_t *rul;
    __device__ __forceinline__ void operator()(size_t r, uint32_t pre, uint32_t v) const
    {
        if (v) rul[pre] = (uint32_t)r;
    }
};

// Pass 1: next ruler and distance from each ruler along LF.  The ruler
// whose successor is ruler 0 ends the chain (no successor; its weight is
// the last hop back to row 0).
__global__ void k_walk_count(const uint32_t *LF, const uint32_t *rul, uint32_t m, uint32_t rows, uint32_t *succ,
                             uint64_t *wt, uint32_t *flags)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    uint32_t r = rul[j], steps = 0, v;
    for (;;) {
        v = __ldg(LF + r);
        steps++;
        if ((v & UB_RULER) || steps > rows) break;
        r = v;
    }
    if (steps > rows) atomicOr(flags, ERR_INTERNAL);
    const uint32_t nx = v & ~UB_RULER;
    succ[j] = nx == 0 ? UB_NIL : nx;
    wt[j] = steps;
}

// Pointer jumping (list ranking): after r rounds wt[j] is the distance over
// the next 2^r rulers (or to the chain's end).  Double-buffered; `open`
// counts rulers that still have a successor.
__global__ void k_jump(const uint32_t *succ, const uint64_t *wt, uint32_t m, uint32_t *succ2, uint64_t *wt2,
                       uint32_t *open)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    const uint32_t s = succ[j];
    if (s == UB_NIL) {
        succ2[j] = UB_NIL;
        wt2[j] = wt[j];
        return;
    }
    wt2[j] = wt[j] + wt[s];
    const uint32_t s2 = succ[s];
    succ2[j] = s2;
    if (s2 != UB_NIL) atomicAdd(open, 1u);
}

// Offsets from row 0: off[j] = total - (distance from ruler j to the end).
__global__ void k_ruler_off(const uint64_t *wt, uint32_t m, uint32_t *off)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    off[j] = (uint32_t)(wt[0] - wt[j]);
}

// Pass 2: every ruler writes the text bytes of its stretch.  sym(row) is
// the bucket of LF(row)-1 among the cumulative symbol counts cum[0..256].
__global__ void k_walk_emit(const uint32_t *LF, const uint32_t *rul, const uint32_t *off, uint32_t m,
                            const uint32_t *cum, uint32_t n, uint8_t *T)
{
    __shared__ uint32_t s_cum[257];
    for (int c = threadIdx.x; c < 257; c += blockDim.x) s_cum[c] = cum[c];
    __syncthreads();
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    uint32_t r = rul[j], k = off[j];
    for (uint32_t s = 0; s <= n; s++, k++) {
        const uint32_t v = __ldg(LF + r);
        const bool last = (v & UB_RULER) != 0;
        const uint32_t t = last ? rul[v & ~UB_RULER] : v;
        if (k < n && t > 0) {
            uint32_t lo = 0, hi = 255;           // last c with cum[c] <= t-1
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1u) >> 1;
                if (s_cum[mid] <= t - 1u) lo = mid; else hi = mid - 1u;
            }
            T[n - 1u - k] = (uint8_t)lo;
        }
        if (last) break;
        r = t;
    }
}

// Cumulative symbol counts: the scanned tile histogram's first tile entries.
__global__ void k_unbwt_cum(const uint32_t *tile_off, uint32_t num_tiles, uint32_t n, uint32_t *cum)
{
    const uint32_t c = threadIdx.x;
    cum[c] = tile_off[(size_t)c * num_tiles];
    if (c == 0) cum[256] = n;
}

void pfp_to_libcubwt(Storage *st, const uint8_t *dO, uint32_t n, uint32_t p, uint8_t *dLc)
{
    k_pfp_to_libcubwt<<<grid_for(n, 256), 256, 0, st->stream>>>(dO, n, p, dLc);
    after_launch(st);
}

// Inverse of libcubwt's convention: Lc (n bytes, device), primary index i in [1, n].
void run_unbwt(Storage *st, const uint8_t *dLc, uint32_t n, uint32_t i, uint8_t *dT)
{
    const uint32_t rows = n + 1u;
    // ~1/128 of the rows are rulers (tuning knob): the longest walk (about
    // rate * ln m steps of one dependent load each) sets the time of both
    // walk passes; small inputs use denser rulers
    const uint32_t rate_max = 1u << tune_unbwt_rate_log2(st);
    uint32_t rate = 4;
    while (rate < rate_max && (uint64_t)rate * 65536u < rows) rate <<= 1;
    const uint32_t rate_mask = rate - 1u;
    // rulers in row order
    check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
    uint32_t *rul = slot<uint32_t>(st, S_SA, rows / 2 + 1024);
    device_scan<uint32_t, OpAdd>(st, rows, LoadRuler{rate_mask}, StoreRuler{rul}, false, (uint32_t *)st->d_scalars);
    fetch_scalars(st, 1);
    const uint32_t m = (uint32_t)st->h_scalars[0];
    if (m == 0 || m > rows / 2 + 1024 || m >= UB_RULER) throw Error{GBWT_INTERNAL_ERROR};
    // LF
    const uint32_t num_tiles = (uint32_t)(((size_t)n + RS_TILE - 1) / RS_TILE);
    uint32_t *hist = slot<uint32_t>(st, S_RSHIST, (size_t)256 * num_tiles);
    k_rs_upsweep<uint8_t, 8><<<num_tiles, RS_THREADS, 0, st->stream>>>(dLc, n, 0, 0xFFu, hist, num_tiles, nullptr);
    after_launch(st);
    scan_array_excl<uint32_t, OpAdd>(st, hist, (size_t)256 * num_tiles, 0);
    uint32_t *LF = slot<uint32_t>(st, S_ISA, rows);
    k_lf_rank<8><<<num_tiles, RS_THREADS, 0, st->stream>>>(dLc, n, i, hist, num_tiles, rate_mask, rul, m, LF);
    after_launch(st);
    uint32_t *cum = slot<uint32_t>(st, S_TMP2, 257);
    k_unbwt_cum<<<1, 256, 0, st->stream>>>(hist, num_tiles, n, cum);
    after_launch(st);
    // walk 1 and list ranking of the ruler chain
    uint32_t *succ = slot<uint32_t>(st, S_TMP0, m), *succ2 = slot<uint32_t>(st, S_TMP1, m);
    uint64_t *wt = slot<uint64_t>(st, S_KEY0, m), *wt2 = slot<uint64_t>(st, S_KEY1, m);
    k_walk_count<<<grid_for(m, 128), 128, 0, st->stream>>>(LF, rul, m, rows, succ, wt, st->d_flags);
    after_launch(st);
    // one list of m rulers closes after ceil(log2 m) rounds; anything still
    // open then lies on a cycle that does not pass row 0
    const int rounds = bits_for(m) + 1;
    for (int r = 0; r < rounds; r++) {
        if (r == rounds - 1) check_cuda(cudaMemsetAsync(st->d_flags + 4, 0, 4, st->stream));
        k_jump<<<grid_for(m, 256), 256, 0, st->stream>>>(succ, wt, m, succ2, wt2, st->d_flags + 4);
        after_launch(st);
        uint32_t *ts = succ; succ = succ2; succ2 = ts;
        uint64_t *tw = wt; wt = wt2; wt2 = tw;
    }
    check_cuda(cudaMemcpyAsync(st->h_scalars + 1, st->d_flags + 4, 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaMemcpyAsync(st->h_scalars + 2, wt, 8, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaMemcpyAsync(st->h_scalars + 3, st->d_flags, 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    if ((uint32_t)st->h_scalars[3] & ERR_INTERNAL) throw Error{GBWT_INTERNAL_ERROR};
    if ((uint32_t)st->h_scalars[1] != 0) throw Error{GBWT_BAD_PARAMETER};
    // from ruler 0 the whole cycle must come back to row 0 after n+1 steps
    if (st->h_scalars[2] != (uint64_t)rows) throw Error{GBWT_BAD_PARAMETER};
    uint32_t *off = slot<uint32_t>(st, S_VAL0, m);
    k_ruler_off<<<grid_for(m, 256), 256, 0, st->stream>>>(wt, m, off);
    after_launch(st);
    k_walk_emit<<<grid_for(m, 128), 128, 0, st->stream>>>(LF, rul, off, m, cum, n, dT);
    after_launch(st);
}

}  // namespace gbwt
