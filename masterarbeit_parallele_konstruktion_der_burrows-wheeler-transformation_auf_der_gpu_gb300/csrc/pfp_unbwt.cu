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
//          rulers (row 0 always); one thread per ruler follows LF to the
//          next ruler (bit 31 of an LF entry marks a ruler target) and
//          records the distance; the host ranks the short ruler chain; a
//          second walk writes every text byte.  The symbol of a row comes
//          from the bucket its LF value falls in, so a step reads one word.
// Walks end at the next ruler; the rulers split the single LF cycle, so the
// steps of all walks sum to n+1.  A BWT whose LF has more than one cycle is
// rejected (the chain of rulers does not cover them all).
#include "prims.cuh"
#include <vector>

namespace gbwt {

constexpr uint32_t UB_RULER = 0x80000000u;

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

// LF of every row.  Element e of Lc is row e (e < i) or e+1 (e >= i).
template <int BITS>
__global__ void __launch_bounds__(RS_THREADS) k_lf_rank(const uint8_t *__restrict__ Lc, uint32_t n, uint32_t i,
                                                        const uint32_t *__restrict__ tile_off, uint32_t num_tiles,
                                                        uint32_t rate_mask, uint32_t *__restrict__ LF)
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
        const uint32_t d = dg[q];
        const bool valid = d != 0xFFFFFFFFu;
        const uint32_t dd = valid ? d : 0u;
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t prior = wh[dd];
        __syncwarp();
        rk[q] = prior + (uint32_t)__popc(peers & ((1u << lane) - 1u));
        if (valid) wh[dd] = prior + (uint32_t)__popc(peers);
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
        LF[row] = t | (ub_is_ruler(t, rate_mask) ? UB_RULER : 0u);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) LF[i] = 0u | UB_RULER;     // '$' row -> row 0
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

// Pass 1: distance from each ruler to the next one along LF.
__global__ void k_walk_count(const uint32_t *LF, const uint32_t *rul, uint32_t m, uint32_t rows, uint32_t *nxt,
                             uint32_t *dist, uint32_t *flags)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    uint32_t r = rul[j], steps = 0, v;
    do {
        v = __ldg(LF + r);
        r = v & ~UB_RULER;
        steps++;
    } while (!(v & UB_RULER) && steps <= rows);
    if (steps > rows) atomicOr(flags, ERR_INTERNAL);
    uint32_t lo = 0, hi = m - 1u;            // ruler index of row r
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (rul[mid] < r) lo = mid + 1u; else hi = mid;
    }
    if (rul[lo] != r) atomicOr(flags, ERR_INTERNAL);
    nxt[j] = lo;
    dist[j] = steps;
}

// Pass 2: every ruler writes the text bytes of its stretch.  sym(row) is
// the bucket of LF(row)-1 among the cumulative symbol counts cum[0..256].
__global__ void k_walk_emit(const uint32_t *LF, const uint32_t *rul, const uint32_t *off, const uint32_t *dist,
                            uint32_t m, const uint32_t *cum, uint32_t n, uint8_t *T)
{
    __shared__ uint32_t s_cum[257];
    for (int c = threadIdx.x; c < 257; c += blockDim.x) s_cum[c] = cum[c];
    __syncthreads();
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= m) return;
    uint32_t r = rul[j], k = off[j];
    const uint32_t steps = dist[j];
    for (uint32_t s = 0; s < steps; s++, k++) {
        const uint32_t v = __ldg(LF + r);
        const uint32_t t = v & ~UB_RULER;
        if (k < n && t > 0) {
            uint32_t lo = 0, hi = 255;           // last c with cum[c] <= t-1
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1u) >> 1;
                if (s_cum[mid] <= t - 1u) lo = mid; else hi = mid - 1u;
            }
            T[n - 1u - k] = (uint8_t)lo;
        }
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
    uint32_t rate = 16;
    while (rate < (1u << 20) && (uint64_t)rate * 262144u < rows) rate <<= 1;
    const uint32_t rate_mask = rate - 1u;
    const uint32_t num_tiles = (uint32_t)(((size_t)n + RS_TILE - 1) / RS_TILE);
    uint32_t *hist = slot<uint32_t>(st, S_RSHIST, (size_t)256 * num_tiles);
    k_rs_upsweep<uint8_t, 8><<<num_tiles, RS_THREADS, 0, st->stream>>>(dLc, n, 0, 0xFFu, hist, num_tiles, nullptr);
    after_launch(st);
    scan_array_excl<uint32_t, OpAdd>(st, hist, (size_t)256 * num_tiles, 0);
    uint32_t *LF = slot<uint32_t>(st, S_ISA, rows);
    k_lf_rank<8><<<num_tiles, RS_THREADS, 0, st->stream>>>(dLc, n, i, hist, num_tiles, rate_mask, LF);
    after_launch(st);
    uint32_t *cum = slot<uint32_t>(st, S_TMP2, 257);
    k_unbwt_cum<<<1, 256, 0, st->stream>>>(hist, num_tiles, n, cum);
    after_launch(st);
    // rulers in row order
    check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
    uint32_t *rul = slot<uint32_t>(st, S_SA, rows / 2 + 1024);
    device_scan<uint32_t, OpAdd>(st, rows, LoadRuler{rate_mask}, StoreRuler{rul}, false, (uint32_t *)st->d_scalars);
    fetch_scalars(st, 1);
    const uint32_t m = (uint32_t)st->h_scalars[0];
    if (m == 0 || m > rows / 2 + 1024) throw Error{GBWT_INTERNAL_ERROR};
    uint32_t *nxt = slot<uint32_t>(st, S_TMP0, m);
    uint32_t *dist = slot<uint32_t>(st, S_TMP1, m);
    uint32_t *off = slot<uint32_t>(st, S_VAL0, m);
    k_walk_count<<<grid_for(m, 128), 128, 0, st->stream>>>(LF, rul, m, rows, nxt, dist, st->d_flags);
    after_launch(st);
    // rank the ruler chain on the host (m is about rows / rate)
    if (st->h_meta_cap < (size_t)3 * m) {
        if (st->h_meta) check_cuda(cudaFreeHost(st->h_meta));
        st->h_meta = nullptr;
        st->h_meta_cap = 0;
        const size_t cap = (size_t)3 * m + 1024;
        check_cuda(cudaHostAlloc(&st->h_meta, cap * sizeof(uint32_t), cudaHostAllocDefault));
        st->h_meta_cap = cap;
    }
    uint32_t *hn = st->h_meta, *hd = st->h_meta + m, *ho = st->h_meta + 2 * (size_t)m;
    check_cuda(cudaMemcpyAsync(hn, nxt, (size_t)m * 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaMemcpyAsync(hd, dist, (size_t)m * 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaMemcpyAsync(st->h_scalars + 1, st->d_flags, 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    if ((uint32_t)st->h_scalars[1] & ERR_INTERNAL) throw Error{GBWT_INTERNAL_ERROR};
    uint64_t acc = 0;
    uint32_t cur = 0;                     // ruler 0 is row 0 (rulers are in row order)
    for (uint32_t it = 0; it < m; it++) {
        if (it > 0 && cur == 0) throw Error{GBWT_BAD_PARAMETER};   // LF has more than one cycle
        ho[cur] = (uint32_t)acc;
        acc += hd[cur];
        cur = hn[cur];
    }
    if (cur != 0 || acc != rows) throw Error{GBWT_BAD_PARAMETER};
    check_cuda(cudaMemcpyAsync(off, ho, (size_t)m * 4, cudaMemcpyHostToDevice, st->stream));
    k_walk_emit<<<grid_for(m, 128), 128, 0, st->stream>>>(LF, rul, off, dist, m, cum, n, dT);
    after_launch(st);
}

}  // namespace gbwt
