// pfp_scan.cu -- Karp-Rabin trigger scan (phrase ends) for sm_103a.
//
// Semantics follow Compute_D1/D2/D3 of the reference
// (Prefix_Free_Parsing_W=5_P=16_kommentiert.cu, "K", K:443-576):
//   window s (s+W-1 < n) triggers when
//     h(s) = sum_{k<W} T[s+W-1-k] * (2^k mod P)  (mod P)  == 0
//   or when T[s..s+W-1] == T[0..W-1]; window 0 never triggers.
//   D lists the triggering windows' last positions, then n+W-1.
//
// GB300 layout: a tile is 4096 window starts; the 4096+W-1 bytes it needs
// are staged in shared memory with 16-byte loads (a CTA loads several tiles
// before it uses any); every thread pulls its 16 windows (+ W-1 halo) into
// registers with 16-byte shared loads and rolls the hash mod P
// (h(s+1) = 2h(s) - T[s]*2^W + T[s+W]); for W=5, P=16 it hashes four
// windows at once with packed byte arithmetic instead.  The first-word test
// rolls an exact packed register for W <= 8 and a 64-bit polynomial
// fingerprint (verified byte by byte on a hit) for longer windows.  Trigger
// positions are compacted with popc + a CTA scan; the count pass also
// validates the input bytes (K:130-132) without trapping.
#include "prims.cuh"
#include <mutex>

namespace gbwt {

constexpr int TS_THREADS = 256;
constexpr int TS_PER_THREAD = 16;
constexpr int TS_TILE = TS_THREADS * TS_PER_THREAD;
constexpr int TS_MAXW = 64;
constexpr uint64_t FP_BASE = 0x100000001B3ull;

struct ScanArgs {
    const uint8_t *T;
    uint32_t n;
    int W;
    int P;
    uint32_t wW;        // 2^W mod P
    uint32_t hi;        // largest valid byte (254, or 15 for the small alphabet)
    uint32_t *flags;    // error bits
};

__device__ __forceinline__ uint32_t bget(const uint32_t *w, int i) { return (w[i >> 2] >> (8 * (i & 3))) & 0xFFu; }

// 2^W mod P: a compile-time constant in the specialised kernels (0 for
// W=5, P=16, where the outgoing byte drops out of the rolling hash).
__host__ __device__ constexpr uint32_t pow2_mod(int W, int P)
{
    uint32_t v = 1;
    for (int i = 0; i < W; i++) v = (v * 2u) % (uint32_t)P;
    return v;
}

// Byte checks of one thread's 16 bytes (K:130-132) on whole 32-bit words.
__device__ __forceinline__ void check_words(const uint32_t *w, uint32_t hi, bool &bad, bool &small_bad)
{
    // a byte b is < 2 iff b & 0xFE is 0, is 255 iff ~b is 0; lane zero test:
    // ~(((v & 0x7F..) + 0x7F..) | v | 0x7F..) sets the lane's top bit
    uint32_t b = 0, sb = 0;
#pragma unroll
    for (int q = 0; q < TS_PER_THREAD / 4; q++) {
        const uint32_t lo = w[q] & 0xFEFEFEFEu, inv = ~w[q];
        b |= ~(((lo & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | lo | 0x7F7F7F7Fu);
        b |= ~(((inv & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | inv | 0x7F7F7F7Fu);
        if (hi == 15u) sb |= w[q] & 0xF0F0F0F0u;
        else if (hi < 254u) sb |= __vcmpgtu4(w[q], hi * 0x01010101u);
    }
    bad = (b & 0x80808080u) != 0;
    small_bad = sb != 0;
}

// Stage bytes [base, base + TS_TILE + W - 1) of T into s (zero past n).
__device__ __forceinline__ void stage_tile(const ScanArgs &a, uint8_t *s, size_t base, int halo16)
{
    const bool aligned = (((uintptr_t)a.T) & 15u) == 0;
    const int nvec = TS_TILE / 16 + halo16;
    for (int v = threadIdx.x; v < nvec; v += TS_THREADS) {
        size_t p = base + (size_t)v * 16;
        uint4 val;
        if (aligned && p + 16 <= a.n) {
            val = __ldg((const uint4 *)(a.T + p));
        } else {
            uint8_t b[16];
#pragma unroll
            for (int j = 0; j < 16; j++) b[j] = (p + j < a.n) ? __ldg(a.T + p + j) : 0;
            memcpy(&val, b, 16);
        }
        *(uint4 *)(s + (size_t)v * 16) = val;
    }
}

// One tile: returns this thread's 16-bit trigger mask and checks bytes.
template <int WT, int PT>
__device__ __forceinline__ uint32_t tile_triggers(const ScanArgs &a, const uint8_t *s, const uint8_t *s_fw,
                                                  uint64_t fw_packed, uint64_t fp0, uint64_t fp_pow,
                                                  size_t base, bool check_bytes)
{
    constexpr int NB = TS_PER_THREAD + (WT > 0 ? WT : TS_MAXW) - 1;   // bytes needed
    constexpr int NV = (NB + 15) / 16;                                 // uint4 loads
    const int W = WT > 0 ? WT : a.W;
    const uint32_t P = PT > 0 ? (uint32_t)PT : (uint32_t)a.P;
    const size_t s0 = base + (size_t)threadIdx.x * TS_PER_THREAD;

    uint32_t w[NV * 4];
    const uint8_t *src = s + (size_t)threadIdx.x * TS_PER_THREAD;
#pragma unroll
    for (int v = 0; v < NV; v++) {
        uint4 q = *(const uint4 *)(src + v * 16);
        w[v * 4 + 0] = q.x; w[v * 4 + 1] = q.y; w[v * 4 + 2] = q.z; w[v * 4 + 3] = q.w;
    }

    if (check_bytes) {
        bool bad = false, small_bad = false;
        if (s0 + TS_PER_THREAD <= a.n) {
            check_words(w, a.hi, bad, small_bad);
        } else {
#pragma unroll
            for (int j = 0; j < TS_PER_THREAD; j++) {
                uint32_t c = bget(w, j);
                if (s0 + j < a.n) {
                    bad |= (c < 2u) || (c == 255u);
                    small_bad |= (c > a.hi);
                }
            }
        }
        if (bad) atomicOr(a.flags, ERR_BAD_BYTE);
        else if (small_bad) atomicOr(a.flags, ERR_SMALL_RANGE);
    }

    if (a.n < (uint32_t)W) return 0;
    const size_t last_valid = (size_t)a.n - (size_t)W;   // last window start
    if (s0 > last_valid) return 0;
    // windows j of this thread that may trigger: s0+j >= 1 and s0+j <= last_valid
    uint32_t range = (last_valid - s0 >= (size_t)TS_PER_THREAD - 1) ? 0xFFFFu
                                                                    : (1u << (uint32_t)(last_valid - s0 + 1)) - 1u;
    if (s0 == 0) range &= ~1u;

    if constexpr (WT == 5 && PT == 16) {
        // Packed byte arithmetic, four windows per 32-bit word.  Window s
        // hashes 8 T[s+1] + 4 T[s+2] + 2 T[s+3] + T[s+4] (mod 16): the weight
        // of T[s] is 2^4 = 0 mod 16.  Each term reduced mod 16 before its
        // shift keeps every byte lane below 64, so one 32-bit add serves four
        // windows.  The first-word test is an OR of byte-wise XORs with the
        // broadcast first five bytes.  A lane is zero exactly when
        // ~(((v & 0x7F..) + 0x7F..) | v | 0x7F..) has its top bit set.
        uint32_t f[5];
#pragma unroll
        for (int k = 0; k < 5; k++) f[k] = (uint32_t)s_fw[k] * 0x01010101u;
        uint32_t m = 0;
#pragma unroll
        for (int q = 0; q < TS_PER_THREAD / 4; q++) {
            const uint32_t x0 = w[q], x4 = w[q + 1];
            const uint32_t x1 = __funnelshift_r(x0, x4, 8);
            const uint32_t x2 = __funnelshift_r(x0, x4, 16);
            const uint32_t x3 = __funnelshift_r(x0, x4, 24);
            const uint32_t hsum = (((x1 & 0x01010101u) << 3) + ((x2 & 0x03030303u) << 2) +
                                   ((x3 & 0x07070707u) << 1) + (x4 & 0x0F0F0F0Fu)) & 0x0F0F0F0Fu;
            const uint32_t e = (x0 ^ f[0]) | (x1 ^ f[1]) | (x2 ^ f[2]) | (x3 ^ f[3]) | (x4 ^ f[4]);
            const uint32_t zh = ~(((hsum & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | hsum | 0x7F7F7F7Fu);
            const uint32_t ze = ~(((e & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | e | 0x7F7F7F7Fu);
            // lane top bits (bits 7, 15, 23, 31) -> four mask bits
            const uint32_t lanes = ((zh | ze) >> 7) & 0x01010101u;
            m |= ((lanes * 0x00204081u) >> 21 & 0xFu) << (4 * q);
        }
        return m & range;
    }

    // hash of the first window: sum b[i] * 2^(W-1-i) mod P
    uint32_t h = 0;
    {
        uint32_t pw = 1;
        uint32_t acc = 0;
#pragma unroll
        for (int i = (WT > 0 ? WT : TS_MAXW) - 1; i >= 0; i--) {
            if (WT == 0 && i >= W) continue;
            acc += bget(w, i) * pw;
            pw = (pw * 2u) % P;
            if (WT == 0 || WT > 16) acc %= P;
        }
        h = acc % P;
    }
    // first-word test state
    uint64_t reg = 0, fp = 0;
    if (WT > 0 && WT <= 8) {
#pragma unroll
        for (int i = 0; i < (WT > 0 ? WT : 1); i++) reg = (reg << 8) | bget(w, i);
    } else {
#pragma unroll
        for (int i = 0; i < (WT > 0 ? WT : TS_MAXW); i++) {
            if (WT == 0 && i >= W) break;
            fp = fp * FP_BASE + bget(w, i);
        }
    }
    const uint64_t regmask = (WT > 0 && WT < 8) ? ((1ull << (8 * (WT > 0 ? WT : 1))) - 1ull) : ~0ull;

    const uint32_t wW = (WT > 0 && PT > 0) ? pow2_mod(WT > 0 ? WT : 1, PT > 0 ? PT : 1) : a.wW;
    uint32_t mask = 0;
#pragma unroll
    for (int j = 0; j < TS_PER_THREAD; j++) {
        const size_t sj = s0 + j;
        bool eq;
        if (WT > 0 && WT <= 8) {
            eq = reg == fw_packed;
        } else {
            eq = false;
            if (fp == fp0) {
                eq = true;
                for (int i = 0; i < W; i++)
                    if (s[sj - base + i] != s_fw[i]) { eq = false; break; }
            }
        }
        if (h == 0 || eq) mask |= 1u << j;
        if (j + 1 < TS_PER_THREAD) {
            const uint32_t out = bget(w, j), in = bget(w, j + W);
            h = (2u * h + in + 256u * P - out * wW) % P;
            if (WT > 0 && WT <= 8) reg = ((reg << 8) | in) & regmask;
            else fp = fp * FP_BASE - (uint64_t)out * fp_pow + in;
        }
    }
    return mask & range;
}

// SUB consecutive 4096-window tiles per CTA: all of their bytes are loaded
// before any is used, so more bytes are in flight per SM than with one tile
// (the scan is otherwise latency-bound on its load).  Trigger order is tile
// by tile, thread by thread: the write pass scans the SUB per-thread counts as
// 16-bit lanes of one 64-bit value.
template <int WT, int PT, bool WRITE, int SUB>
__global__ void __launch_bounds__(TS_THREADS) k_trigger(ScanArgs a, uint32_t *counts, const uint32_t *offsets,
                                                        uint32_t *D)
{
    static_assert(SUB >= 1 && SUB <= 4, "the write pass packs SUB counts into 16-bit lanes");
    __shared__ __align__(16) uint8_t s[SUB * TS_TILE + TS_MAXW + 64];
    __shared__ uint8_t s_fw[TS_MAXW];
    __shared__ uint64_t s_warp[32];
    const int W = WT > 0 ? WT : a.W;
    const size_t base = (size_t)blockIdx.x * (SUB * TS_TILE);
    const int halo16 = (W - 1 + 15) / 16 + 1;
    {
        // the CTA's SUB tiles, one 16-byte vector per thread and tile, all
        // loads issued first; then the halo past the last tile
        const bool aligned = (((uintptr_t)a.T) & 15u) == 0;
        uint4 v[SUB];
#pragma unroll
        for (int k = 0; k < SUB; k++) {
            const size_t p = base + ((size_t)k * TS_THREADS + threadIdx.x) * 16;
            if (aligned && p + 16 <= a.n) {
                v[k] = __ldg((const uint4 *)(a.T + p));
            } else {
                uint8_t bb[16];
#pragma unroll
                for (int j = 0; j < 16; j++) bb[j] = (p + j < a.n) ? __ldg(a.T + p + j) : 0;
                memcpy(&v[k], bb, 16);
            }
        }
#pragma unroll
        for (int k = 0; k < SUB; k++) *(uint4 *)(s + ((size_t)k * TS_THREADS + threadIdx.x) * 16) = v[k];
        for (int h = threadIdx.x; h < halo16; h += TS_THREADS) {
            const size_t p = base + (size_t)SUB * TS_TILE + (size_t)h * 16;
            uint4 val;
            if (aligned && p + 16 <= a.n) {
                val = __ldg((const uint4 *)(a.T + p));
            } else {
                uint8_t bb[16];
#pragma unroll
                for (int j = 0; j < 16; j++) bb[j] = (p + j < a.n) ? __ldg(a.T + p + j) : 0;
                memcpy(&val, bb, 16);
            }
            *(uint4 *)(s + (size_t)SUB * TS_TILE + (size_t)h * 16) = val;
        }
    }
    if (threadIdx.x < (unsigned)W) s_fw[threadIdx.x] = threadIdx.x < a.n ? __ldg(a.T + threadIdx.x) : 1;
    __syncthreads();

    uint64_t fw_packed = 0, fp0 = 0, fp_pow = 1;
    for (int i = 0; i < W; i++) {
        fw_packed = (fw_packed << 8) | s_fw[i];
        fp0 = fp0 * FP_BASE + s_fw[i];
        fp_pow *= FP_BASE;
    }
    uint32_t mask[SUB];
    uint64_t packed = 0;
#pragma unroll
    for (int k = 0; k < SUB; k++) {
        mask[k] = tile_triggers<WT, PT>(a, s + (size_t)k * TS_TILE, s_fw, fw_packed, fp0, fp_pow,
                                         base + (size_t)k * TS_TILE, !WRITE);
        packed |= (uint64_t)__popc(mask[k]) << (16 * k);
    }
    uint64_t total;
    const uint64_t ex = block_excl_scan<uint64_t, OpAdd>(packed, total, OpAdd(), s_warp);
    if (!WRITE) {
        if (threadIdx.x == 0) {
            uint32_t c = 0;
#pragma unroll
            for (int k = 0; k < SUB; k++) c += (uint32_t)(total >> (16 * k)) & 0xFFFFu;
            counts[blockIdx.x] = c;
        }
        return;
    }
    uint32_t tile_base = offsets[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SUB; k++) {
        uint32_t o = tile_base + ((uint32_t)(ex >> (16 * k)) & 0xFFFFu);
        const uint32_t s0 = (uint32_t)(base + (size_t)k * TS_TILE + (size_t)threadIdx.x * TS_PER_THREAD);
        uint32_t m = mask[k];
        while (m) {
            const int j = __ffs(m) - 1;
            m &= m - 1;
            D[o++] = s0 + (uint32_t)j + (uint32_t)W - 1u;
        }
        tile_base += (uint32_t)(total >> (16 * k)) & 0xFFFFu;
    }
}

constexpr int TS_SUB = 4;      // tiles per CTA in the pipeline's scan

template <int WT, int PT>
static void launch_pair(Storage *st, const ScanArgs &a, unsigned blocks, uint32_t *counts, uint32_t *&D)
{
    probe_begin(st, GBWT_PROBE_TRIGGER_SCAN);
    k_trigger<WT, PT, false, TS_SUB><<<blocks, TS_THREADS, 0, st->stream>>>(a, counts, nullptr, nullptr);
    probe_end(st, GBWT_PROBE_TRIGGER_SCAN, a.n);
    after_launch(st);
    // exclusive scan of block counts; total -> d_scalars[0]
    uint32_t *tot = (uint32_t *)st->d_scalars;
    check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
    device_scan<uint32_t, OpAdd>(st, blocks, LoadArr<uint32_t>{counts}, StoreArr<uint32_t>{counts}, false, tot);
    check_cuda(cudaMemcpyAsync(st->h_scalars + 1, a.flags, 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaMemcpyAsync(st->h_scalars, st->d_scalars, 8, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    uint32_t flags = (uint32_t)st->h_scalars[1];
    if (flags & ERR_BAD_BYTE) throw Error{GBWT_BAD_PARAMETER};
    if (flags & ERR_SMALL_RANGE) throw Error{GBWT_UNSUPPORTED_INPUT};
    uint32_t c = (uint32_t)(st->h_scalars[0] & 0xFFFFFFFFu);
    D = slot<uint32_t>(st, S_D, (size_t)c + 1);
    probe_begin(st, GBWT_PROBE_TRIGGER_SCAN);
    k_trigger<WT, PT, true, TS_SUB><<<blocks, TS_THREADS, 0, st->stream>>>(a, nullptr, counts, D);
    probe_end(st, GBWT_PROBE_TRIGGER_SCAN, (uint64_t)a.n + 4ull * c);
    after_launch(st);
    k_set_u32<<<1, 1, 0, st->stream>>>(D + c, a.n + (uint32_t)a.W - 1u);
    after_launch(st);
    st->h_scalars[0] = c;
}

uint32_t run_trigger_scan(Storage *st, const uint8_t *dT, uint32_t n, int W, int P, bool small, uint32_t *&D)
{
    ScanArgs a;
    a.T = dT; a.n = n; a.W = W; a.P = P;
    uint32_t wW = 1;
    for (int i = 0; i < W; i++) wW = (wW * 2u) % (uint32_t)P;
    a.wW = wW;
    a.hi = small ? 15u : 254u;
    a.flags = st->d_flags;
    unsigned blocks = grid_for(n, TS_TILE * TS_SUB);
    uint32_t *counts = slot<uint32_t>(st, S_TMP0, blocks + 1);
    if (W == 5 && P == 16) launch_pair<5, 16>(st, a, blocks, counts, D);
    else if (W == 5 && P == 11) launch_pair<5, 11>(st, a, blocks, counts, D);
    else if (W == 5 && P == 13) launch_pair<5, 13>(st, a, blocks, counts, D);
    else if (W == 5 && P == 14) launch_pair<5, 14>(st, a, blocks, counts, D);
    else if (W == 5 && P == 23) launch_pair<5, 23>(st, a, blocks, counts, D);
    else if (W == 35 && P == 81) launch_pair<35, 81>(st, a, blocks, counts, D);
    else launch_pair<0, 0>(st, a, blocks, counts, D);
    return (uint32_t)st->h_scalars[0] + 1u;
}

// ---------------------------------------------------------------------
// Batched trigger scan over a padded buffer X of many texts: text t at
// xstart[t] followed by W sentinel bytes (1).  Per text the windows are
// those of its own scan (start s >= 1 inside the text, s+W-1 < n_t), and
// the text's forced final trigger is the all-sentinel window right after it.
// Both tests read only X: the W+1 bytes X[s-1 .. s+W-1] hold no sentinel
// for an ordinary window, and exactly W (all but X[s-1]) for the forced one.
// The first-window rule compares with the first window of the window's own
// text, whose index is the number of text starts up to s, minus one.
// ---------------------------------------------------------------------
struct BatchScanArgs {
    const uint32_t *tile_text;   // [tiles] text starts before each tile
    const uint64_t *fw;          // [k] first window of each text (packed, or fingerprint)
    const uint32_t *xstart;      // [k] text starts in X
};

// First windows: packed big-endian bytes for W <= 8, else the fingerprint
// used by the scan (both as computed by tile_triggers).
__global__ void k_first_words(const uint8_t *X, const uint32_t *xstart, uint32_t k, int W, uint64_t *fw)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= k) return;
    const uint8_t *p = X + xstart[t];
    uint64_t v = 0;
    if (W <= 8) {
        for (int i = 0; i < W; i++) v = (v << 8) | p[i];
    } else {
        for (int i = 0; i < W; i++) v = v * FP_BASE + p[i];
    }
    fw[t] = v;
}

// tile_text[b] = number of text starts below b * TS_TILE.
__global__ void k_tile_text(const uint32_t *xstart, uint32_t k, uint32_t tiles, uint32_t *tile_text)
{
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= tiles) return;
    const uint32_t base = b * (uint32_t)TS_TILE;
    uint32_t lo = 0, hi = k;        // first index with xstart >= base
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (xstart[mid] < base) lo = mid + 1; else hi = mid;
    }
    tile_text[b] = lo;
}

template <int WT, int PT>
__device__ __forceinline__ uint32_t tile_triggers_batch(const ScanArgs &a, const BatchScanArgs &b, const uint8_t *s,
                                                        uint32_t prevb, size_t base, uint32_t tcur, uint64_t fp_pow)
{
    constexpr int NB = TS_PER_THREAD + (WT > 0 ? WT : TS_MAXW) - 1;
    constexpr int NV = (NB + 15) / 16;
    const int W = WT > 0 ? WT : a.W;
    const uint32_t P = PT > 0 ? (uint32_t)PT : (uint32_t)a.P;
    const size_t s0 = base + (size_t)threadIdx.x * TS_PER_THREAD;
    if (s0 >= a.n) return 0;

    uint32_t w[NV * 4];
    const uint8_t *src = s + (size_t)threadIdx.x * TS_PER_THREAD;
#pragma unroll
    for (int v = 0; v < NV; v++) {
        uint4 q = *(const uint4 *)(src + v * 16);
        w[v * 4 + 0] = q.x; w[v * 4 + 1] = q.y; w[v * 4 + 2] = q.z; w[v * 4 + 3] = q.w;
    }
    uint32_t h = 0, c1 = prevb == 1u;
    {
        uint32_t pw = 1, acc = 0;
#pragma unroll
        for (int i = (WT > 0 ? WT : TS_MAXW) - 1; i >= 0; i--) {
            if (WT == 0 && i >= W) continue;
            const uint32_t c = bget(w, i);
            acc += c * pw;
            c1 += c == 1u;
            pw = (pw * 2u) % P;
            if (WT == 0 || WT > 16) acc %= P;
        }
        h = acc % P;
    }
    uint64_t reg = 0, fp = 0;
    if (WT > 0 && WT <= 8) {
#pragma unroll
        for (int i = 0; i < (WT > 0 ? WT : 1); i++) reg = (reg << 8) | bget(w, i);
    } else {
#pragma unroll
        for (int i = 0; i < (WT > 0 ? WT : TS_MAXW); i++) {
            if (WT == 0 && i >= W) break;
            fp = fp * FP_BASE + bget(w, i);
        }
    }
    const uint64_t regmask = (WT > 0 && WT < 8) ? ((1ull << (8 * (WT > 0 ? WT : 1))) - 1ull) : ~0ull;
    const uint32_t wW = (WT > 0 && PT > 0) ? pow2_mod(WT > 0 ? WT : 1, PT > 0 ? PT : 1) : a.wW;
    uint64_t cur = tcur ? __ldg(b.fw + tcur - 1) : 0ull;

    // Almost every thread sees no sentinel byte, neither just before its
    // windows nor in them: no text starts there, no window is forced, and
    // the test is the single-text one against a fixed first window.
    const uint32_t nb = (uint32_t)TS_PER_THREAD + (uint32_t)W - 1u;
    bool clean = prevb != 1u && s0 + nb <= a.n;
    if (clean) {
        uint32_t ones = 0;
#pragma unroll
        for (int q = 0; q < NV * 4; q++) {
            if ((uint32_t)q * 4u >= nb) break;
            uint32_t m = __vcmpeq4(w[q], 0x01010101u);
            if (nb - (uint32_t)q * 4u < 4u) m &= (1u << (8u * (nb - (uint32_t)q * 4u))) - 1u;
            ones |= m;
        }
        clean = ones == 0;
    }
    uint32_t mask = 0;
    if (clean) {
#pragma unroll
        for (int j = 0; j < TS_PER_THREAD; j++) {
            bool eq;
            if (WT > 0 && WT <= 8) {
                eq = reg == cur;
            } else {
                eq = false;
                if (fp == cur) {
                    const uint8_t *f = a.T + __ldg(b.xstart + tcur - 1);
                    eq = true;
                    for (int i = 0; i < W; i++)
                        if (s[s0 + j - base + i] != __ldg(f + i)) { eq = false; break; }
                }
            }
            if (h == 0 || eq) mask |= 1u << j;
            if (j + 1 < TS_PER_THREAD) {
                const uint32_t out = bget(w, j), in = bget(w, j + W);
                h = (2u * h + in + 256u * P - out * wW) % P;
                if (WT > 0 && WT <= 8) reg = ((reg << 8) | in) & regmask;
                else fp = fp * FP_BASE - (uint64_t)out * fp_pow + in;
            }
        }
        return mask;
    }
#pragma unroll
    for (int j = 0; j < TS_PER_THREAD; j++) {
        const size_t sj = s0 + j;
        const uint32_t pb = j ? bget(w, j - 1) : prevb, c = bget(w, j);
        const bool inside = sj < a.n;
        if (inside && pb == 1u && c != 1u) {          // a text starts at sj
            tcur++;
            cur = __ldg(b.fw + tcur - 1);
        }
        if (inside) {
            bool hit = false;
            if (c1 == 0) {
                bool eq;
                if (WT > 0 && WT <= 8) {
                    eq = reg == cur;
                } else {
                    eq = false;
                    if (fp == cur) {
                        const uint8_t *f = a.T + __ldg(b.xstart + tcur - 1);
                        eq = true;
                        for (int i = 0; i < W; i++)
                            if (s[sj - base + i] != __ldg(f + i)) { eq = false; break; }
                    }
                }
                hit = h == 0 || eq;
            } else {
                hit = pb != 1u && c1 == (uint32_t)W;   // forced end of the text
            }
            if (hit) mask |= 1u << j;
        }
        if (j + 1 < TS_PER_THREAD) {
            const uint32_t in = bget(w, j + W);
            h = (2u * h + in + 256u * P - c * wW) % P;
            c1 += (in == 1u) - (pb == 1u);
            if (WT > 0 && WT <= 8) reg = ((reg << 8) | in) & regmask;
            else fp = fp * FP_BASE - (uint64_t)c * fp_pow + in;
        }
    }
    return mask;
}

template <int WT, int PT, bool WRITE>
__global__ void __launch_bounds__(TS_THREADS) k_trigger_batch(ScanArgs a, BatchScanArgs b, uint32_t *counts,
                                                              const uint32_t *offsets, uint32_t *D)
{
    __shared__ __align__(16) uint8_t s[TS_TILE + TS_MAXW + 64];
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_prev;
    const int W = WT > 0 ? WT : a.W;
    const size_t base = (size_t)blockIdx.x * TS_TILE;
    const int halo16 = (W - 1 + 15) / 16 + 1;
    stage_tile(a, s, base, halo16);
    if (threadIdx.x == 0) s_prev = base ? __ldg(a.T + base - 1) : 1u;
    __syncthreads();
    // text starts among this thread's 16 positions -> text count before s0
    const uint32_t o = threadIdx.x * TS_PER_THREAD;
    const uint32_t prevb = threadIdx.x ? s[o - 1] : s_prev;
    uint32_t nst = 0;
    const uint4 q4 = *(const uint4 *)(s + o);
    const uint32_t ones = __vcmpeq4(q4.x, 0x01010101u) | __vcmpeq4(q4.y, 0x01010101u) |
                          __vcmpeq4(q4.z, 0x01010101u) | __vcmpeq4(q4.w, 0x01010101u);
    if (prevb == 1u || ones) {        // a text can only start after a sentinel byte
        uint32_t pb = prevb;
#pragma unroll
        for (int j = 0; j < TS_PER_THREAD; j++) {
            const uint32_t c = s[o + j];
            nst += (base + o + j < a.n && pb == 1u && c != 1u) ? 1u : 0u;
            pb = c;
        }
    }
    uint32_t tot;
    const uint32_t ex_st = block_excl_scan<uint32_t, OpAdd>(nst, tot, OpAdd(), s_warp);
    const uint32_t tcur = __ldg(b.tile_text + blockIdx.x) + ex_st;
    __syncthreads();
    uint64_t fp_pow = 1;
    for (int i = 0; i < W; i++) fp_pow *= FP_BASE;
    uint32_t mask = tile_triggers_batch<WT, PT>(a, b, s, prevb, base, tcur, fp_pow);
    uint32_t cnt = __popc(mask), total;
    uint32_t ex = block_excl_scan<uint32_t, OpAdd>(cnt, total, OpAdd(), s_warp);
    if (!WRITE) {
        if (threadIdx.x == 0) counts[blockIdx.x] = total;
        return;
    }
    uint32_t out = offsets[blockIdx.x] + ex;
    const uint32_t s0 = (uint32_t)(base + o);
    while (mask) {
        int j = __ffs(mask) - 1;
        mask &= mask - 1;
        D[out++] = s0 + (uint32_t)j + (uint32_t)W - 1u;
    }
}

template <int WT, int PT>
static uint32_t launch_pair_batch(Storage *st, const ScanArgs &a, const BatchScanArgs &b, unsigned blocks,
                                  uint32_t *counts, uint32_t *&D)
{
    probe_begin(st, GBWT_PROBE_TRIGGER_SCAN);
    k_trigger_batch<WT, PT, false><<<blocks, TS_THREADS, 0, st->stream>>>(a, b, counts, nullptr, nullptr);
    probe_end(st, GBWT_PROBE_TRIGGER_SCAN, a.n);
    after_launch(st);
    uint32_t *tot = (uint32_t *)st->d_scalars;
    check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
    device_scan<uint32_t, OpAdd>(st, blocks, LoadArr<uint32_t>{counts}, StoreArr<uint32_t>{counts}, false, tot);
    check_cuda(cudaMemcpyAsync(st->h_scalars + 1, a.flags, 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaMemcpyAsync(st->h_scalars, st->d_scalars, 8, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    const uint32_t flags = (uint32_t)st->h_scalars[1];
    if (flags & ERR_BAD_BYTE) throw Error{GBWT_BAD_PARAMETER};
    if (flags & ERR_SMALL_RANGE) throw Error{GBWT_UNSUPPORTED_INPUT};
    const uint32_t c = (uint32_t)(st->h_scalars[0] & 0xFFFFFFFFu);
    D = slot<uint32_t>(st, S_D, (size_t)c + 1);
    probe_begin(st, GBWT_PROBE_TRIGGER_SCAN);
    k_trigger_batch<WT, PT, true><<<blocks, TS_THREADS, 0, st->stream>>>(a, b, nullptr, counts, D);
    probe_end(st, GBWT_PROBE_TRIGGER_SCAN, (uint64_t)a.n + 4ull * c);
    after_launch(st);
    return c;
}

uint32_t run_trigger_scan_batch(Storage *st, const uint8_t *dX, uint32_t N, int W, int P, const uint32_t *xstart,
                                uint32_t k, uint32_t *&D)
{
    ScanArgs a;
    a.T = dX; a.n = N; a.W = W; a.P = P;
    uint32_t wW = 1;
    for (int i = 0; i < W; i++) wW = (wW * 2u) % (uint32_t)P;
    a.wW = wW;
    a.hi = 254u;             // bytes were checked when X was built
    a.flags = st->d_flags;
    const unsigned blocks = grid_for(N, TS_TILE);
    uint32_t *counts = slot<uint32_t>(st, S_TMP0, blocks + 1);
    uint32_t *tile_text = slot<uint32_t>(st, S_TMP1, blocks);
    uint64_t *fw = slot<uint64_t>(st, S_TMP2, k);
    k_first_words<<<grid_for(k, 256), 256, 0, st->stream>>>(dX, xstart, k, W, fw);
    after_launch(st);
    k_tile_text<<<grid_for(blocks, 256), 256, 0, st->stream>>>(xstart, k, blocks, tile_text);
    after_launch(st);
    BatchScanArgs b{tile_text, fw, xstart};
    if (W == 5 && P == 16) return launch_pair_batch<5, 16>(st, a, b, blocks, counts, D);
    if (W == 5 && P == 23) return launch_pair_batch<5, 23>(st, a, b, blocks, counts, D);
    if (W == 35 && P == 81) return launch_pair_batch<35, 81>(st, a, b, blocks, counts, D);
    return launch_pair_batch<0, 0>(st, a, b, blocks, counts, D);
}

// ---------------------------------------------------------------------
// Allocation-free trigger scan.
//
// Some callers cannot allocate device memory themselves: code running
// under a fixed memory budget handed out by a host framework, an allocator
// that must not be re-entered from a callback, or a process that pins all
// device memory up front.  For them the trigger scan also runs without a
// storage object and without any cudaMalloc: its scratch (per-CTA trigger
// counts, the scan's tile partials, the error/total words) lives in the
// file-scope array below, which every GPU that loads this library holds
// until the process exits (NOALLOC_SCRATCH_WORDS * 4 bytes, about 1 MiB).
// Texts are limited to NOALLOC_MAX_N bytes by that size.  All calls share
// the array: calls whose work overlaps on the GPU (other streams, other host
// threads) race on it and must be serialised by the caller.
// ---------------------------------------------------------------------
constexpr int64_t NOALLOC_MAX_N = (int64_t)1 << 30;
constexpr uint32_t NOALLOC_MAX_BLOCKS = (uint32_t)(NOALLOC_MAX_N / TS_TILE);
constexpr uint32_t NOALLOC_PARTIALS = (NOALLOC_MAX_BLOCKS + SC_TILE - 1) / SC_TILE;
constexpr uint32_t NOALLOC_SCRATCH_WORDS = NOALLOC_MAX_BLOCKS + 256 + 64;

static __device__ __align__(256) uint32_t g_trigger_scratch[NOALLOC_SCRATCH_WORDS];

// Device address of g_trigger_scratch for the current device, looked up
// once per device (the host-side symbol itself is not a device address).
// The same first call checks the compute capability, so an unsupported GPU
// gets GBWT_GPU_NOT_SUPPORTED before any work is queued on the caller's
// stream (the kernels are built for sm_103a only).
static uint32_t *noalloc_scratch_ptr()
{
    static uint32_t *ptrs[64] = {};
    static std::mutex mu;
    int dev = 0;
    check_cuda(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw Error{GBWT_GPU_NOT_SUPPORTED};
    std::lock_guard<std::mutex> lock(mu);
    if (!ptrs[dev]) {
        int major = 0, minor = 0;
        check_cuda(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
        check_cuda(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
        if (major * 10 + minor != 103) throw Error{GBWT_GPU_NOT_SUPPORTED};
        void *p = nullptr;
        check_cuda(cudaGetSymbolAddress(&p, g_trigger_scratch));
        ptrs[dev] = (uint32_t *)p;
    }
    return ptrs[dev];
}

template <int WT, int PT>
static int64_t noalloc_launch(const ScanArgs &a, unsigned blocks, uint32_t *scratch, uint32_t *D, int64_t capacity,
                              cudaStream_t stream)
{
    uint32_t *counts = scratch;                         // [NOALLOC_MAX_BLOCKS]
    uint32_t *partials = scratch + NOALLOC_MAX_BLOCKS;  // [256]
    uint32_t *words = partials + 256;                   // [0] errors, [1] trigger count
    check_cuda(cudaMemsetAsync(words, 0, 64 * sizeof(uint32_t), stream));
    ScanArgs b = a;
    b.flags = words;
    k_trigger<WT, PT, false, 1><<<blocks, TS_THREADS, 0, stream>>>(b, counts, nullptr, nullptr);
    check_cuda(cudaGetLastError());
    const unsigned tiles = (blocks + SC_TILE - 1) / SC_TILE;
    if (tiles == 1) {
        k_scan_down<uint32_t, OpAdd><<<1, SC_THREADS, 0, stream>>>(LoadArr<uint32_t>{counts}, StoreArr<uint32_t>{counts},
                                                                    blocks, (const uint32_t *)nullptr, false, words + 1);
    } else {
        k_scan_reduce<uint32_t, OpAdd><<<tiles, SC_THREADS, 0, stream>>>(LoadArr<uint32_t>{counts}, blocks, partials);
        k_scan_down<uint32_t, OpAdd><<<1, SC_THREADS, 0, stream>>>(LoadArr<uint32_t>{partials},
                                                                    StoreArr<uint32_t>{partials}, tiles,
                                                                    (const uint32_t *)nullptr, false, (uint32_t *)nullptr);
        k_scan_down<uint32_t, OpAdd><<<tiles, SC_THREADS, 0, stream>>>(LoadArr<uint32_t>{counts},
                                                                        StoreArr<uint32_t>{counts}, blocks, partials,
                                                                        false, words + 1);
    }
    check_cuda(cudaGetLastError());
    uint32_t host_words[2] = {0, 0};
    check_cuda(cudaMemcpyAsync(host_words, words, sizeof(host_words), cudaMemcpyDeviceToHost, stream));
    check_cuda(cudaStreamSynchronize(stream));
    if (host_words[0] & ERR_BAD_BYTE) return GBWT_BAD_PARAMETER;
    if (host_words[0] & ERR_SMALL_RANGE) return GBWT_UNSUPPORTED_INPUT;
    const uint32_t c = host_words[1];
    if ((int64_t)c + 1 > capacity) return GBWT_BAD_PARAMETER;
    k_trigger<WT, PT, true, 1><<<blocks, TS_THREADS, 0, stream>>>(b, nullptr, counts, D);
    k_set_u32<<<1, 1, 0, stream>>>(D + c, a.n + (uint32_t)a.W - 1u);
    check_cuda(cudaGetLastError());
    check_cuda(cudaStreamSynchronize(stream));
    return (int64_t)c + 1;
}

}  // namespace gbwt

extern "C" int64_t gbwt_pfp_trigger_scan_noalloc(const uint8_t *T, int64_t n, int32_t W, int32_t P, uint32_t flags,
                                                 uint32_t *D, int64_t capacity, void *stream)
{
    using namespace gbwt;
    if (n < 0 || n > NOALLOC_MAX_N || W < 1 || W > 64 || P < 1 || P > 65535) return GBWT_BAD_PARAMETER;
    if (n == 0) return 0;
    if (!T || !D || capacity < 1) return GBWT_BAD_PARAMETER;
    try {
        uint32_t *scratch = noalloc_scratch_ptr();
        ScanArgs a;
        a.T = T; a.n = (uint32_t)n; a.W = W; a.P = P;
        uint32_t wW = 1;
        for (int i = 0; i < W; i++) wW = (wW * 2u) % (uint32_t)P;
        a.wW = wW;
        a.hi = (flags & GBWT_FLAG_SMALL_ALPHABET) ? 15u : 254u;
        a.flags = nullptr;
        const unsigned blocks = grid_for((size_t)n, TS_TILE);
        cudaStream_t s = (cudaStream_t)stream;
        if (W == 5 && P == 16) return noalloc_launch<5, 16>(a, blocks, scratch, D, capacity, s);
        if (W == 5 && P == 11) return noalloc_launch<5, 11>(a, blocks, scratch, D, capacity, s);
        if (W == 5 && P == 13) return noalloc_launch<5, 13>(a, blocks, scratch, D, capacity, s);
        if (W == 5 && P == 14) return noalloc_launch<5, 14>(a, blocks, scratch, D, capacity, s);
        if (W == 5 && P == 23) return noalloc_launch<5, 23>(a, blocks, scratch, D, capacity, s);
        if (W == 35 && P == 81) return noalloc_launch<35, 81>(a, blocks, scratch, D, capacity, s);
        return noalloc_launch<0, 0>(a, blocks, scratch, D, capacity, s);
    } catch (const Error &e) {
        return e.code;
    }
}
