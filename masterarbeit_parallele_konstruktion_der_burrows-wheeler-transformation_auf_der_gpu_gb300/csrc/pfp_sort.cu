// pfp_sort.cu -- prefix doubling with discarding (sm_103a), used twice:
//
//  1. Dictionary order.  Every position of the concatenated distinct
//     phrases is sorted by the phrase suffix that starts there (suffixes
//     end at their phrase end).  This one sort yields the lexicographic
//     phrase ranks (positions at offset 0) that the reference obtains with
//     its per-byte MSD sort of all occurrences (K:1990-2164), and the order
//     of the suffix set S that it sorts separately (K:4408-4552).  Groups of
//     equal suffixes stay tied, which is how S deduplicates.
//  2. Parse suffix array, the reference's Sort_Suffix_Array (K:2342-2412):
//     prefix doubling over (rank_i, rank_{i+h}) keys, discarding resolved
//     groups.
//
// "K" is Prefix_Free_Parsing_W=5_P=16_kommentiert.cu of the reference.
//
// Invariant of round h: isa[x] is the first sorted position of x's group of
// equal h-prefixes; groups are finished when they are singletons or when
// their common string ends within h symbols.  Every group is uniform in
// whether its strings end within h symbols: the initial keys encode it
// (dictionary: an explicit bit; parse: the unique last phrase), and a round
// keyed on isa[x+h] inherits it from the groups of x+h.
//
// Round 0 sorts the first keys with the stable LSD radix sort and derives
// group heads and the active list in one packed scan (the single-text parse
// instead takes its first ranks straight from the phrase buckets).  Every
// later round gathers isa[x+h] for the active elements and sorts each group
// by it inside a CTA (k_seg_sort); the few groups too large for a CTA take
// one radix sort of their members only.
#include "prims.cuh"
#include <stdio.h>
#include <stdlib.h>
#include <algorithm>
#include <vector>

namespace gbwt {

// Remaining length of the suffix at x (rem(x)) and the test ends(x, h) =
// rem(x) <= h: the suffix is fully compared once its first h symbols are.
// Dictionary suffixes end with their phrase; rem8[x] = min(rem(x), 255) (one
// byte per position, L2-resident) answers ends() for h < 255 without the
// phrase-table lookups.
struct DictRem {
    const uint32_t *dphr, *doff, *dlen;
    const uint8_t *rem8;
    __device__ __forceinline__ uint32_t operator()(uint32_t x) const
    {
        uint32_t q = dphr[x];
        return doff[q] + dlen[q] - x;
    }
    __device__ __forceinline__ bool ends(uint32_t x, uint32_t h) const
    {
        if (rem8 && h < 255u) return rem8[x] <= h;
        return (*this)(x) <= h;
    }
};

struct ParseRem {
    uint32_t n;
    __device__ __forceinline__ uint32_t operator()(uint32_t x) const { return n - x; }
    __device__ __forceinline__ bool ends(uint32_t x, uint32_t h) const { return n - x <= h; }
};
// A batch of parses laid end to end: a suffix ends with its own text; the
// remaining length of every suffix is precomputed.  ends(x, h) first asks a
// bitmap of 64-position blocks holding a text's last position (L1-sized):
// when no block of [x, x+h-1] holds one, the text of x goes on past x+h-1
// and the remaining length is not loaded.
constexpr uint32_t BR_MAPH = 1024;      // longest range the bitmap answers
struct BatchParseRem {
    const uint32_t *remv;
    const uint32_t *endmap;
    __device__ __forceinline__ uint32_t operator()(uint32_t x) const { return remv[x]; }
    __device__ __forceinline__ bool ends(uint32_t x, uint32_t h) const
    {
        if (h == 0) return false;
        if (h <= BR_MAPH && x <= 0xFFFFFFFFu - BR_MAPH) {
            const uint32_t b0 = x >> 6, b1 = (x + h - 1u) >> 6;       // b1 - b0 <= 16
            const uint32_t w0 = b0 >> 5, w1 = b1 >> 5;
            uint32_t m = __ldg(endmap + w0) >> (b0 & 31u);
            if (w0 == w1) {
                m &= 0xFFFFFFFFu >> (31u - (b1 - b0));
            } else if (!m) {
                m = __ldg(endmap + w1) & (0xFFFFFFFFu >> (31u - (b1 & 31u)));
            }
            if (!m) return false;
        }
        return remv[x] <= h;
    }
};
__global__ void k_batch_rem(const uint32_t *ptid, const uint32_t *zend, uint32_t z, uint32_t *remv)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x < z) remv[x] = zend[ptid[x]] - x;
}
// Bit b of endmap: some text's last parse position lies in [64b, 64b+64).
__global__ void k_text_endmap(const uint32_t *zend, uint32_t k, uint32_t *endmap)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= k) return;
    const uint32_t e = zend[t] - 1u;
    atomicOr(endmap + (e >> 11), 1u << ((e >> 6) & 31u));
}

__global__ void k_iota(uint32_t *v, uint32_t n)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

// Active test after a round whose prefix length is now `h`.
template <typename Rem>
struct ActiveTest {
    const uint64_t *k;
    const uint32_t *vals;
    uint32_t n;
    uint32_t h;
    Rem rem;
    __device__ __forceinline__ bool done(size_t t) const
    {
        const uint64_t key = k[t];
        const bool single = (t == 0 || k[t - 1] != key) && (t + 1 == n || k[t + 1] != key);
        return single || rem.ends(vals[t], h);
    }
};

template <typename Rem>
struct LoadActive {
    ActiveTest<Rem> a;
    __device__ __forceinline__ uint32_t operator()(size_t t) const { return a.done(t) ? 0u : 1u; }
};
// Round 0 after the sort, in one scan of packed pairs: the high word is a
// max-scan of group starts (an element's group head), the low word counts
// the active elements before it (its slot in the active list).  Finished
// elements go straight to their suffix-array slot t.
template <typename Rem>
struct LoadHeadActive0 {
    ActiveTest<Rem> a;
    bool cont_bit;      // key bit 0 = "suffix longer than the key's symbols": no rem() gather
    __device__ __forceinline__ uint64_t operator()(size_t t) const
    {
        const uint64_t key = a.k[t];
        const bool first = t == 0 || a.k[t - 1] != key;
        const bool last = t + 1 == a.n || a.k[t + 1] != key;
        const bool done = (first && last) || (cont_bit ? (key & 1u) == 0 : a.rem.ends(a.vals[t], a.h));
        return ((uint64_t)(first ? (uint32_t)t : 0u) << 32) | (done ? 0u : 1u);
    }
};
template <typename Rem>
struct StoreHeadActive0 {
    ActiveTest<Rem> a;
    uint32_t *isa;
    uint32_t *sa;
    uint32_t *act_x;
    uint32_t *act_g;
    __device__ __forceinline__ void operator()(size_t t, uint64_t pre, uint64_t v) const
    {
        const uint32_t x = a.vals[t];
        const uint32_t ph = (uint32_t)(pre >> 32), vh = (uint32_t)(v >> 32);
        const uint32_t h = ph > vh ? ph : vh;          // inclusive max: the group head
        isa[x] = h;
        if ((uint32_t)v) {
            act_x[(uint32_t)pre] = x;
            act_g[(uint32_t)pre] = h;
        } else {
            sa[t] = x;
        }
    }
};

// Packed max-scan: high word = start of the old group, low = start of the new group.
struct LoadRoundHead {
    const uint64_t *k;
    int lb;
    __device__ __forceinline__ uint64_t operator()(size_t a) const
    {
        const uint64_t key = k[a];
        bool gnew = a == 0 || (k[a - 1] >> lb) != (key >> lb);
        bool knew = a == 0 || k[a - 1] != key;
        return (gnew ? ((uint64_t)a << 32) : 0ull) | (knew ? (uint64_t)a : 0ull);
    }
};
// ---------------------------------------------------------------------
// Segmented round for small groups.  After the first rounds almost every
// group is small (a repetitive text's copies of one position), so a CTA
// sorts whole groups in shared memory instead of running global radix
// passes.  CTA b owns the groups that start in active indices
// [b*SS_TILE, (b+1)*SS_TILE); a group may run past the tile by at most
// SS_SEGMAX elements, so a CTA holds < SS_TILE + SS_SEGMAX elements.
// ---------------------------------------------------------------------
constexpr int SS_THREADS = 512;
constexpr int SS_TILE = 2048;
constexpr int SS_SEGMAX = 2048;
constexpr int SS_CAP = SS_TILE + SS_SEGMAX;
constexpr int SS_PER_THREAD = SS_CAP / SS_THREADS;
constexpr uint32_t SS_WARPMAX = 256;      // larger groups are sorted by the CTA
constexpr uint32_t SS_COUNTMAX = 12;      // smaller groups rank by counting, unsorted
constexpr int SS_MISC_WORDS = 8 + 64 + 16; // misc, scan scratch (32 x u64), big-group list
constexpr int SS_MIDMAX = SS_CAP / (SS_COUNTMAX + 1) + 1;   // groups above SS_COUNTMAX in one CTA
// keys, x, segment heads, segment starts, slot heads (4 B each), misc,
// element -> segment and slot -> element (2 B each), warp-group list (2 B)
constexpr size_t SS_SMEM = (size_t)SS_CAP * (8 + 4 + 4 + 4 + 4 + 2 + 2) + SS_MISC_WORDS * 4 + SS_MIDMAX * 2;
// two CTAs per SM (228 KB of shared memory, 1 KB reserved per CTA)
static_assert(2 * (SS_SMEM + 1024) <= 228 * 1024, "k_seg_sort must keep two CTAs per SM");
// a group of at most SS_SEGMAX members cannot cover a whole tile, so every
// full tile after the first group start holds a group start
static_assert(SS_SEGMAX <= SS_TILE, "tile starts need groups no longer than a tile");

// Sorts key[0..s) ascending with a bitonic network whose merge steps start
// with the "flipped" comparator (i, block_end-1-i): every comparator is
// ascending, so the virtual padding to a power of two (positions >= s, seen
// as +infinity) never moves and needs no storage.  Run by `nthr` threads
// (a warp, or the whole CTA when `cta`).
__device__ __forceinline__ void bitonic_flip_sort(uint64_t *key, uint32_t s, uint32_t tid, uint32_t nthr, bool cta)
{
    if (s < 2) return;
    uint32_t lgh = 0;                       // log2(k/2)
    for (uint32_t k = 2; (k >> 1) < s; k <<= 1, lgh++) {
        for (uint32_t p = tid; p < (s + 1) / 2 + k / 2; p += nthr) {
            const uint32_t blk = p >> lgh, r = p & ((k >> 1) - 1);
            const uint32_t i = blk * k + r, l = blk * k + k - 1 - r;
            if (l < s) {
                const uint64_t a = key[i], b = key[l];
                if (a > b) { key[i] = b; key[l] = a; }
            }
        }
        if (cta) __syncthreads(); else __syncwarp();
        for (uint32_t jj = k >> 2; jj > 0; jj >>= 1) {
            for (uint32_t p = tid; p < (s + 1) / 2 + jj; p += nthr) {
                const uint32_t i = 2 * p - (p & (jj - 1)), l = i + jj;
                if (l < s) {
                    const uint64_t a = key[i], b = key[l];
                    if (a > b) { key[i] = b; key[l] = a; }
                }
            }
            if (cta) __syncthreads(); else __syncwarp();
        }
    }
}

// Warp sort of key[0..s), s <= 32*E, in registers: E keys per lane in
// blocked order (element lane*E+e), +infinity padding, bitonic network with
// in-lane compare-exchanges for distances < E and shfl_xor across lanes for
// the others.
template <int E>
__device__ __forceinline__ void warp_sort_regs(uint64_t *key, uint32_t s, uint32_t lane)
{
    constexpr uint32_t N = 32u * E;
    uint64_t v[E];
#pragma unroll
    for (int e = 0; e < E; e++) {
        const uint32_t i = lane * E + e;
        v[e] = i < s ? key[i] : ~0ull;
    }
#pragma unroll
    for (uint32_t k = 2; k <= N; k <<= 1) {
#pragma unroll
        for (uint32_t j = k >> 1; j > 0; j >>= 1) {
            if (j >= (uint32_t)E) {
#pragma unroll
                for (int e = 0; e < E; e++) {
                    const uint32_t i = lane * E + e;
                    const uint64_t o = __shfl_xor_sync(0xFFFFFFFFu, v[e], j / E);
                    const bool asc = (i & k) == 0, lower = (i & j) == 0;
                    v[e] = (lower == asc) ? (v[e] < o ? v[e] : o) : (v[e] > o ? v[e] : o);
                }
            } else {
#pragma unroll
                for (int e = 0; e < E; e++) {
                    if ((e & j) == 0) {
                        const int e2 = e | (int)j;
                        const uint32_t i = lane * E + e;
                        const bool asc = (i & k) == 0;
                        if ((v[e] > v[e2]) == asc) { const uint64_t t = v[e]; v[e] = v[e2]; v[e2] = t; }
                    }
                }
            }
        }
    }
#pragma unroll
    for (int e = 0; e < E; e++) {
        const uint32_t i = lane * E + e;
        if (i < s) key[i] = v[e];
    }
    __syncwarp();
}

// One group of s members (13..): keys key[0..s) = (isa[x+h]+1) << 32 | local
// index li, xs[li] = the member's suffix.  Writes, for every sorted slot p,
// nh[p] = new group head | done bit and perm[p] = li.  Run by one warp.
template <typename Rem>
__device__ __forceinline__ void warp_group(uint64_t *key, uint32_t s, uint32_t g, const uint32_t *xs, uint32_t h2,
                                           const Rem &rem, uint32_t *out_nh, uint16_t *out_perm, uint32_t lane,
                                           bool collect_stats, uint32_t *flags)
{
    // Fast paths (groups of a repetitive text's copies): the next ranks
    // isa[x+h] of a group usually take one value, two values, or one
    // majority value with a few outliers.  A stable partition in input
    // order replaces the sort.  One counting pass first: min, max, and
    // for two candidate values (middle and first member) their counts
    // and the number of members below them.
    const uint32_t c1 = (uint32_t)(key[s >> 1] >> 32), c2 = (uint32_t)(key[0] >> 32);
    uint32_t mn = 0xFFFFFFFFu, mx = 0, n1 = 0, n2 = 0, b1 = 0, b2 = 0;
    for (uint32_t c0 = 0; c0 < s; c0 += 32) {
        const uint32_t i = c0 + lane;
        const bool in = i < s;
        const uint32_t k2 = in ? (uint32_t)(key[i] >> 32) : c1;
        if (in) {
            mn = min(mn, k2);
            mx = max(mx, k2);
        }
        n1 += __popc(__ballot_sync(0xFFFFFFFFu, in && k2 == c1));
        n2 += __popc(__ballot_sync(0xFFFFFFFFu, in && k2 == c2));
        b1 += __popc(__ballot_sync(0xFFFFFFFFu, in && k2 < c1));
        b2 += __popc(__ballot_sync(0xFFFFFFFFu, in && k2 < c2));
    }
    mn = __reduce_min_sync(0xFFFFFFFFu, mn);
    mx = __reduce_max_sync(0xFFFFFFFFu, mx);
    const uint32_t mj = n1 >= n2 ? c1 : c2, ne = n1 >= n2 ? n1 : n2, nl = n1 >= n2 ? b1 : b2;
    if (collect_stats && lane == 0)
        atomicAdd(flags + 20 + (mn == mx ? 0 : (s - ne <= 32 ? 3 : 2)), s);
    if (s <= SS_WARPMAX && s - ne <= 32) {
        // majority members in input order after the nl smaller ones;
        // outlier j goes to lane j and is ranked by counting
        uint64_t mine = ~0ull;
        uint32_t no = 0, re = 0;
        for (uint32_t c0 = 0; c0 < s; c0 += 32) {
            const uint32_t i = c0 + lane;
            const bool in = i < s;
            const uint64_t kk = in ? key[i] : 0ull;
            const bool me = in && (uint32_t)(kk >> 32) == mj;
            const unsigned be = __ballot_sync(0xFFFFFFFFu, me);
            const unsigned bo = __ballot_sync(0xFFFFFFFFu, in && !me);
            if (me) {
                const uint32_t pos = nl + re + __popc(be & ((1u << lane) - 1u));
                const uint32_t li = (uint32_t)kk & 0xFFFFu;
                const bool done = ne == 1 || rem.ends(xs[li], h2);
                out_nh[pos] = (g + nl) | (done ? 0x80000000u : 0u);
                out_perm[pos] = (uint16_t)li;
            }
            re += __popc(be);
            if (bo) {
                const uint32_t want = lane - no;      // this chunk's outlier for this lane
                const bool take = lane >= no && want < (uint32_t)__popc(bo);
                const uint32_t src = take ? (uint32_t)__fns(bo, 0, (int)want + 1) : lane;
                const uint64_t got = __shfl_sync(0xFFFFFFFFu, kk, src);
                if (take) mine = got;
                no += __popc(bo);
            }
        }
        const uint32_t my2 = (uint32_t)(mine >> 32);
        uint32_t rk = 0, lt2 = 0, eq2 = 0;
        for (uint32_t q = 0; q < no; q++) {
            const uint64_t o = __shfl_sync(0xFFFFFFFFu, mine, q);
            const uint32_t o2 = (uint32_t)(o >> 32);
            rk += o < mine;
            lt2 += o2 < my2;
            eq2 += o2 == my2;
        }
        if (lane < no) {
            const bool above = my2 > mj;
            const uint32_t pos = above ? rk + ne : rk;
            const uint32_t li = (uint32_t)mine & 0xFFFFu;
            const bool done = eq2 == 1 || rem.ends(xs[li], h2);
            out_nh[pos] = (g + (above ? lt2 + ne : lt2)) | (done ? 0x80000000u : 0u);
            out_perm[pos] = (uint16_t)li;
        }
        return;
    }
    // exactly two values, both frequent: stable two-way partition
    bool two = false;
    uint32_t cmn = 0;                    // members with the smaller value
    {
        bool other = false;
        for (uint32_t c0 = 0; c0 < s; c0 += 32) {
            const uint32_t i = c0 + lane;
            const uint32_t k2 = i < s ? (uint32_t)(key[i] >> 32) : mn;
            other |= (k2 != mn && k2 != mx);
            cmn += __popc(__ballot_sync(0xFFFFFFFFu, i < s && k2 == mn));
        }
        two = !__any_sync(0xFFFFFFFFu, other);
    }
    if (two) {
        uint32_t rmn = 0, rmx = 0;       // running ranks among equal members
        for (uint32_t c0 = 0; c0 < s; c0 += 32) {
            const uint32_t i = c0 + lane;
            const bool in = i < s;
            const uint32_t k2 = in ? (uint32_t)(key[i] >> 32) : 0u;
            const bool lo = in && k2 == mn;
            const unsigned blo = __ballot_sync(0xFFFFFFFFu, lo), bhi = __ballot_sync(0xFFFFFFFFu, in && !lo);
            const unsigned lt = (1u << lane) - 1u;
            if (in) {
                const uint32_t li = (uint32_t)key[i] & 0xFFFFu;
                uint32_t pos, nh;
                bool single;
                if (lo) { pos = rmn + __popc(blo & lt); nh = g; single = cmn == 1; }
                else { pos = cmn + rmx + __popc(bhi & lt); nh = g + cmn; single = s - cmn == 1; }
                const bool done = single || rem.ends(xs[li], h2);
                out_nh[pos] = nh | (done ? 0x80000000u : 0u);
                out_perm[pos] = (uint16_t)li;
            }
            rmn += __popc(blo);
            rmx += __popc(bhi);
        }
        return;
    }
    if (s <= 32) warp_sort_regs<1>(key, s, lane);
    else if (s <= 64) warp_sort_regs<2>(key, s, lane);
    else if (s <= 128) warp_sort_regs<4>(key, s, lane);
    else if (s <= SS_WARPMAX) warp_sort_regs<8>(key, s, lane);
    // new heads: start of each run of equal key2 (carried across chunks)
    uint32_t carry = 0;
    for (uint32_t c0 = 0; c0 < s; c0 += 32) {
        const uint32_t i = c0 + lane;
        const bool in = i < s;
        const uint64_t kk = in ? key[i] : 0ull;
        const uint32_t k2 = (uint32_t)(kk >> 32);
        const bool knew = in && (i == 0 || (uint32_t)(key[i - 1] >> 32) != k2);
        const unsigned bal = __ballot_sync(0xFFFFFFFFu, knew);
        const unsigned upto = bal & (0xFFFFFFFFu >> (31u - lane));
        const uint32_t gstart = upto ? c0 + 31u - __clz(upto) : carry;
        if (in) {
            const bool single = knew && (i + 1 == s || (uint32_t)(key[i + 1] >> 32) != k2);
            const uint32_t li = (uint32_t)kk & 0xFFFFu;
            const bool done = single || rem.ends(xs[li], h2);
            out_nh[i] = (g + gstart) | (done ? 0x80000000u : 0u);
            out_perm[i] = (uint16_t)li;
        }
        carry = __shfl_sync(0xFFFFFFFFu, gstart, 31);
    }
}

// key2[a] = isa[x+h] + 1 for every active element (all reads of this round's
// ranks happen before any update); tstart[b] = first group start in tile b
// (SS_TILE active indices; 0xFFFFFFFF before, via memset).  With `bigs`,
// groups too large for the shared-memory path (more than SS_SEGMAX members)
// are listed: flags[3] / flags[4] count their starts / ends, bigs[i] = the
// i-th start, bigs[big_cap + i] = the i-th end (one past the last member;
// both lists in no particular order), and tbig[b] = the start of the one that
// starts in tile b (a tile holds at most one: such a group is longer than a
// tile).
__global__ void k_round_gather(const uint32_t *act_x, const uint32_t *act_g, const uint32_t *isa, uint32_t A_arg,
                               const uint32_t *Ap, uint32_t h, uint32_t *key2, uint32_t *flags, uint32_t *tstart,
                               uint32_t *bigs, uint32_t big_cap, uint32_t *tbig, uint32_t *hist)
{
    // the active count: a launch argument when the host knows it, else read
    // on the device (the grid then covers an upper bound)
    const uint32_t A = Ap ? *Ap : A_arg;
    if (hist && blockIdx.x == 0 && threadIdx.x == 0) *hist = A;
    const uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x * blockDim.x >= A) return;
    bool gnew = false;
    if (a < A) {
        key2[a] = isa[act_x[a] + h] + 1u;
        const uint32_t g = act_g[a];
        gnew = a == 0 || act_g[a - 1] != g;
        if (bigs) {
            if (gnew && a + SS_SEGMAX < A && act_g[a + SS_SEGMAX] == g) {
                const uint32_t i = atomicAdd(flags + 3, 1u);
                if (i < big_cap) bigs[i] = a;
                else atomicOr(flags, ERR_INTERNAL);
                tbig[a / SS_TILE] = a;
            }
            const bool gend = a + 1u == A || act_g[a + 1u] != g;
            if (gend && a >= SS_SEGMAX && act_g[a - SS_SEGMAX] == g) {
                const uint32_t i = atomicAdd(flags + 4, 1u);
                if (i < big_cap) bigs[big_cap + i] = a + 1u;
                else atomicOr(flags, ERR_INTERNAL);
            }
        }
    }
    // a block's indices lie in one tile (blockDim divides SS_TILE): one
    // global atomic per block with a group start
    __shared__ uint32_t s_first;
    if (threadIdx.x == 0) s_first = 0xFFFFFFFFu;
    __syncthreads();
    const uint32_t first = __reduce_min_sync(0xFFFFFFFFu, gnew ? a : 0xFFFFFFFFu);
    if ((threadIdx.x & 31u) == 0 && first != 0xFFFFFFFFu) atomicMin(&s_first, first);
    __syncthreads();
    if (threadIdx.x == 0 && s_first != 0xFFFFFFFFu) atomicMin(tstart + s_first / SS_TILE, s_first);
}

template <typename Rem>
__global__ void __launch_bounds__(SS_THREADS, 2) k_seg_sort(const uint32_t *__restrict__ act_x,
                                                            const uint32_t *__restrict__ act_g,
                                                            const uint32_t *__restrict__ key2,
                                                            const uint32_t *__restrict__ tstart,
                                                            const uint32_t *__restrict__ tbig, uint32_t A_arg,
                                                            const uint32_t *__restrict__ Ap, uint32_t h2, Rem rem, uint32_t *isa, uint32_t *sa,
                                                            uint32_t *out_x, uint32_t *out_g, uint32_t *counter,
                                                            uint32_t *flags, bool collect_stats)
{
    extern __shared__ __align__(16) unsigned char ss_smem[];
    uint64_t *s_key = (uint64_t *)ss_smem;           // (isa[x+h]+1) << 32 | local index
    uint32_t *s_x = (uint32_t *)(s_key + SS_CAP);    // local index -> x
    uint32_t *s_sg = s_x + SS_CAP;                   // segment -> group head g
    uint32_t *s_ss = s_sg + SS_CAP;                  // segment -> local start index
    uint32_t *s_nh = s_ss + SS_CAP;                  // sorted slot -> new head | done bit
    uint32_t *s_misc = s_nh + SS_CAP;                // [2] warp counter, [3] big, [4] base, [5] warp groups
    uint64_t *s_scan = (uint64_t *)(s_misc + 8);
    uint32_t *s_big = s_misc + 8 + 64;
    uint16_t *s_seg = (uint16_t *)(s_misc + SS_MISC_WORDS);   // local index -> segment
    uint16_t *s_perm = s_seg + SS_CAP;                        // sorted slot -> local index
    uint16_t *s_mid = s_perm + SS_CAP;                        // segments above SS_COUNTMAX

    // the CTA's elements: from the first group start in its tile to the
    // first group start in the next tile (or A)
    const uint32_t A = Ap ? *Ap : A_arg;             // from the device: the grid covers an upper bound
    const uint32_t tiles = (A + SS_TILE - 1) / SS_TILE;
    if (blockIdx.x >= tiles) return;
    const uint32_t s0 = tstart[blockIdx.x];
    if (s0 == 0xFFFFFFFFu) return;                   // no group starts in this tile
    uint32_t e1;
    const uint32_t bstart = tbig ? tbig[blockIdx.x] : 0xFFFFFFFFu;
    if (bstart != 0xFFFFFFFFu) {
        // a group too large for this path starts in this tile (at or after
        // s0) and runs past it: the range ends there, the big-group path
        // sorts it
        e1 = bstart;
    } else {
        e1 = blockIdx.x + 1 < tiles ? tstart[blockIdx.x + 1] : A;
        if (e1 == 0xFFFFFFFFu) {
            // only the last tile, partly filled, may lack a start
            if (blockIdx.x + 2 < tiles) { if (threadIdx.x == 0) atomicOr(flags, ERR_INTERNAL); return; }
            e1 = A;
        }
    }
    const uint32_t cnt = e1 - s0;
    if (cnt == 0) return;
    if (cnt > (uint32_t)SS_CAP) { if (threadIdx.x == 0) atomicOr(flags, ERR_INTERNAL); return; }

    // coalesced loads into shared memory (s_nh holds the group ids for now)
#pragma unroll
    for (int j = 0; j < SS_PER_THREAD; j++) {
        const uint32_t i = (uint32_t)j * SS_THREADS + threadIdx.x;
        if (i < cnt) {
            const uint32_t a = s0 + i;
            // unique key: (isa[x+h]+1, local index) -- stable, deterministic
            s_key[i] = ((uint64_t)key2[a] << 32) | i;
            s_x[i] = act_x[a];
            s_nh[i] = act_g[a];
        }
    }
    __syncthreads();
    // segments in element order, warp-striped: warp w owns local indices
    // [w*256, w*256+256) as 8 rows of 32 lanes (ballots give the order
    // inside a row; consecutive lanes touch consecutive banks)
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t wb = (threadIdx.x >> 5) * (32u * SS_PER_THREAD);
    const unsigned lt = (1u << lane) - 1u;
    unsigned rowm[SS_PER_THREAD];
    uint32_t wcnt = 0;
#pragma unroll
    for (int j = 0; j < SS_PER_THREAD; j++) {
        const uint32_t i = wb + (uint32_t)j * 32u + lane;
        rowm[j] = __ballot_sync(0xFFFFFFFFu, i < cnt && (i == 0 || s_nh[i - 1] != s_nh[i]));
        wcnt += __popc(rowm[j]);
    }
    uint64_t tot;
    uint32_t run = (uint32_t)block_excl_scan<uint64_t, OpAdd>(lane == 0 ? (uint64_t)wcnt : 0ull, tot, OpAdd(), s_scan);
    run = __shfl_sync(0xFFFFFFFFu, run, 0);
    const uint32_t nsegs = (uint32_t)tot;
#pragma unroll
    for (int j = 0; j < SS_PER_THREAD; j++) {
        const uint32_t i = wb + (uint32_t)j * 32u + lane;
        if (i < cnt) {
            const uint32_t start = (rowm[j] >> lane) & 1u;
            const uint32_t sidx = run + (uint32_t)__popc(rowm[j] & lt) + start - 1u;   // segment of i
            if (start) { s_sg[sidx] = s_nh[i]; s_ss[sidx] = i; }
            s_seg[i] = (uint16_t)sidx;
        }
        run += (uint32_t)__popc(rowm[j]);
    }
    if (threadIdx.x == 0) { s_ss[nsegs] = cnt; s_misc[2] = 0; s_misc[3] = 0; s_misc[5] = 0; }
    __syncthreads();

    // Tier 3: groups larger than SS_WARPMAX are sorted by the whole CTA.
    // flags[16..19] accumulate group statistics per tier (elements in groups
    // <= SS_COUNTMAX, <= SS_WARPMAX, larger; number of groups).
    uint32_t e1c = 0, e2c = 0, e3c = 0;
    for (uint32_t sg = threadIdx.x; sg < nsegs; sg += SS_THREADS) {
        const uint32_t s = s_ss[sg + 1] - s_ss[sg];
        if (s > SS_COUNTMAX) s_mid[atomicAdd(&s_misc[5], 1u)] = (uint16_t)sg;
        if (s > SS_WARPMAX) { s_big[atomicAdd(&s_misc[3], 1u)] = sg; e3c += s; }
        else if (s > SS_COUNTMAX) e2c += s;
        else e1c += s;
    }
    if (collect_stats) {
        e1c = __reduce_add_sync(0xFFFFFFFFu, e1c);
        e2c = __reduce_add_sync(0xFFFFFFFFu, e2c);
        e3c = __reduce_add_sync(0xFFFFFFFFu, e3c);
        if ((threadIdx.x & 31u) == 0) {
            if (e1c) atomicAdd(flags + 16, e1c);
            if (e2c) atomicAdd(flags + 17, e2c);
            if (e3c) atomicAdd(flags + 18, e3c);
        }
        if (threadIdx.x == 0) atomicAdd(flags + 19, nsegs);
    }
    __syncthreads();
    const uint32_t nbig = s_misc[3];
    for (uint32_t b = 0; b < nbig; b++) {
        const uint32_t ss = s_ss[s_big[b]], s = s_ss[s_big[b] + 1] - ss;
        bitonic_flip_sort(s_key + ss, s, threadIdx.x, SS_THREADS, true);
    }

    // Tier 1: groups of at most SS_COUNTMAX elements -- every element counts
    // the smaller keys of its group (no sort at all) and records its slot.
#pragma unroll
    for (int j = 0; j < SS_PER_THREAD; j++) {
        const uint32_t i = (uint32_t)j * SS_THREADS + threadIdx.x;
        if (i >= cnt) break;
        const uint32_t sg = s_seg[i];
        const uint32_t ss = s_ss[sg], se = s_ss[sg + 1];
        if (se - ss > SS_COUNTMAX) continue;
        const uint64_t kk = s_key[i];
        const uint32_t k2 = (uint32_t)(kk >> 32);
        uint32_t lt = 0, eq = 0, pos = 0;
        for (uint32_t m = ss; m < se; m++) {
            const uint64_t o = s_key[m];
            const uint32_t o2 = (uint32_t)(o >> 32);
            lt += o2 < k2;
            eq += o2 == k2;
            pos += o < kk;
        }
        const bool done = eq == 1 || rem.ends(s_x[i], h2);
        s_nh[ss + pos] = (s_sg[sg] + lt) | (done ? 0x80000000u : 0u);
        s_perm[ss + pos] = (uint16_t)i;
    }

    // Tiers 2/3: warps take the larger groups from a shared counter, sort the
    // ones up to SS_WARPMAX, and derive the new heads of all of them.
    const uint32_t nmid = s_misc[5];
    for (;;) {
        uint32_t m = 0;
        if (lane == 0) m = atomicAdd(&s_misc[2], 1u);
        m = __shfl_sync(0xFFFFFFFFu, m, 0);
        if (m >= nmid) break;
        const uint32_t sg = s_mid[m];
        const uint32_t ss = s_ss[sg], se = s_ss[sg + 1], s = se - ss;
        const uint32_t g = s_sg[sg];
        // (groups above SS_WARPMAX were sorted by the CTA above; warp_group
        // derives their heads only)
        warp_group<Rem>(s_key + ss, s, g, s_x, h2, rem, s_nh + ss, s_perm + ss, lane, collect_stats, flags);
    }
    __syncthreads();

    // Final pass over sorted slots: ranks, finished suffixes, and the CTA's
    // share of the next active list (reserved with one atomic; the order of
    // groups in that list does not matter, only each group being contiguous).
    // Active slots are counted warp-striped like the segments above.
    unsigned actm[SS_PER_THREAD];
    uint32_t wact = 0;
#pragma unroll
    for (int j = 0; j < SS_PER_THREAD; j++) {
        const uint32_t p = wb + (uint32_t)j * 32u + lane;
        actm[j] = __ballot_sync(0xFFFFFFFFu, p < cnt && !(s_nh[p] >> 31));
        wact += __popc(actm[j]);
    }
    uint64_t atot;
    uint32_t apre = (uint32_t)block_excl_scan<uint64_t, OpAdd>(lane == 0 ? (uint64_t)wact : 0ull, atot, OpAdd(),
                                                              s_scan);
    apre = __shfl_sync(0xFFFFFFFFu, apre, 0);
    if (threadIdx.x == 0) s_misc[4] = atot ? atomicAdd(counter, (uint32_t)atot) : 0u;
    // active slots (x, new head) staged in slot order; the keys are dead
    uint2 *s_act = (uint2 *)s_key;
#pragma unroll
    for (int j = 0; j < SS_PER_THREAD; j++) {
        const uint32_t p = wb + (uint32_t)j * 32u + lane;
        if ((actm[j] >> lane) & 1u) s_act[apre + (uint32_t)__popc(actm[j] & lt)] = make_uint2(s_x[s_perm[p]], s_nh[p]);
        apre += (uint32_t)__popc(actm[j]);
    }
    __syncthreads();
    const uint32_t base = s_misc[4];
    // striped: ranks, finished suffixes, next active list
    for (uint32_t p = threadIdx.x; p < cnt; p += SS_THREADS) {
        const uint32_t v = s_nh[p];
        const uint32_t nh = v & 0x7FFFFFFFu;
        const uint32_t x = s_x[s_perm[p]];
        const uint32_t sg = s_seg[p];                 // slots stay inside their group
        // isa[x] already holds the old group head (the rank it was made
        // active with); only a changed rank is written
        if (nh != s_sg[sg]) isa[x] = nh;
        if (v >> 31) sa[s_sg[sg] + (p - s_ss[sg])] = x;
    }
    for (uint32_t k = threadIdx.x; k < (uint32_t)atot; k += SS_THREADS) {
        const uint2 e = s_act[k];
        out_x[base + k] = e.x;
        out_g[base + k] = e.y;
    }
}

__global__ void k_big_heads(const uint32_t *act_g, const uint32_t *bstart, uint32_t nbig, uint32_t *bhead)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nbig) bhead[i] = act_g[bstart[i]];
}

// ---------------------------------------------------------------------
// Big-group path.  Groups with more than SS_SEGMAX members (listed by the
// gather, cut out of the segmented kernel's ranges) are sorted together by
// one global radix sort over their members only, keyed (big-group index,
// isa[x+h] + 1); one scan derives the new heads, one scan appends the
// members that stay active to the next active list after the ones the
// segmented kernel wrote.  In a repetitive text only a few groups (frequent
// short phrases, early rounds) take it.
// ---------------------------------------------------------------------
__global__ void k_big_keys(const uint32_t *bstart, const uint32_t *boff, uint32_t nbig, const uint32_t *key2,
                           const uint32_t *act_x, int lb, uint64_t *keys, uint32_t *vals)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t total = boff[nbig];
    if (t >= total) return;
    uint32_t lo = 0, hi = nbig - 1u;                 // last group with boff <= t
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1u) >> 1;
        if (boff[mid] <= t) lo = mid; else hi = mid - 1u;
    }
    const uint32_t a = bstart[lo] + (t - boff[lo]);
    keys[t] = ((uint64_t)lo << lb) | (uint64_t)key2[a];
    vals[t] = act_x[a];
}
template <typename Rem>
struct StoreBigRound {
    ActiveTest<Rem> t;
    int lb;
    const uint32_t *bhead;
    uint32_t *isa;
    uint32_t *head;
    uint32_t *sa;
    __device__ __forceinline__ void operator()(size_t a, uint64_t inc, uint64_t) const
    {
        const uint32_t g = bhead[(uint32_t)(t.k[a] >> lb)];
        const uint32_t ag = (uint32_t)(inc >> 32), s2 = (uint32_t)inc;
        const uint32_t nh = g + (s2 - ag);
        const uint32_t x = t.vals[a];
        if (nh != g) isa[x] = nh;                     // isa[x] holds the old head g
        head[a] = nh;
        if (t.done(a)) sa[g + ((uint32_t)a - ag)] = x;
    }
};
template <typename Rem>
struct StoreBigActive {
    ActiveTest<Rem> a;
    const uint32_t *head;
    const uint32_t *counter;      // elements the segmented kernel appended
    uint32_t *act_x;
    uint32_t *act_g;
    __device__ __forceinline__ void operator()(size_t t, uint32_t pre, uint32_t v) const
    {
        if (v) {
            const uint32_t base = *counter;
            act_x[base + pre] = a.vals[t];
            act_g[base + pre] = head[t];
        }
    }
};

template <typename Rem>
static void big_groups(Storage *st, uint32_t N, uint32_t nbig, const uint32_t *dbigs, uint32_t big_cap, uint32_t h2,
                       const uint32_t *key2, const uint32_t *act_x, const uint32_t *act_g, Rem rem, uint32_t *isa,
                       uint32_t *sa, uint32_t *out_x, uint32_t *out_g, const uint32_t *counter, uint32_t *big_total)
{
    // starts and ends, both sorted: big groups are disjoint ranges, so the
    // i-th start and the i-th end delimit the i-th group
    std::vector<uint32_t> hb(nbig), he(nbig), hoff(nbig + 1);
    check_cuda(cudaMemcpyAsync(hb.data(), dbigs, (size_t)nbig * 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaMemcpyAsync(he.data(), dbigs + big_cap, (size_t)nbig * 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    std::sort(hb.begin(), hb.end());
    std::sort(he.begin(), he.end());
    hoff[0] = 0;
    for (uint32_t i = 0; i < nbig; i++) {
        if (he[i] <= hb[i] + SS_SEGMAX || (i + 1 < nbig && he[i] > hb[i + 1])) throw Error{GBWT_INTERNAL_ERROR};
        hoff[i + 1] = hoff[i] + (he[i] - hb[i]);
    }
    const uint32_t total = hoff[nbig];
    uint32_t *meta = slot<uint32_t>(st, S_BIGM, (size_t)nbig * 3 + 2);   // starts, offsets, heads
    check_cuda(cudaMemcpyAsync(meta, hb.data(), (size_t)nbig * 4, cudaMemcpyHostToDevice, st->stream));
    check_cuda(cudaMemcpyAsync(meta + nbig, hoff.data(), (size_t)(nbig + 1) * 4, cudaMemcpyHostToDevice,
                               st->stream));
    uint32_t *bhead = meta + 2 * nbig + 1;
    k_big_heads<<<grid_for(nbig, 256), 256, 0, st->stream>>>(act_g, meta, nbig, bhead);
    after_launch(st);
    const int lb = bits_for(N);
    uint64_t *k = slot<uint64_t>(st, S_KEY0, total);
    uint64_t *k_alt = slot<uint64_t>(st, S_KEY1, total);
    uint32_t *v = slot<uint32_t>(st, S_VAL0, total);
    uint32_t *v_alt = slot<uint32_t>(st, S_VAL1, total);
    uint32_t *head = slot<uint32_t>(st, S_HEAD, total);
    k_big_keys<<<grid_for(total, 256), 256, 0, st->stream>>>(meta, meta + nbig, nbig, key2, act_x, lb, k, v);
    after_launch(st);
    radix_sort<uint64_t, true>(st, k, k_alt, v, v_alt, total, 0, lb + bits_for(nbig - 1u));
    ActiveTest<Rem> t{k, v, total, h2, rem};
    device_scan<uint64_t, OpMax2>(st, total, LoadRoundHead{k, lb}, StoreBigRound<Rem>{t, lb, bhead, isa, head, sa},
                                  true, (uint64_t *)nullptr);
    check_cuda(cudaMemsetAsync(big_total, 0, 4, st->stream));
    device_scan<uint32_t, OpAdd>(st, total, LoadActive<Rem>{t},
                                 StoreBigActive<Rem>{t, head, counter, out_x, out_g}, false, big_total);
}

__global__ void k_add_u32(uint32_t *dst, const uint32_t *src) { *dst += *src; }
__global__ void k_set_word(uint32_t *dst, uint32_t v) { *dst = v; }

// Prefix-doubling rounds from prefix length h with A active elements listed
// group by group in act_x (suffix) / act_g (group head); isa holds every
// suffix's group head and sa every finished slot.  Returns the rounds run.
//
// The active count of each round stays on the device (two counters used in
// turn: the kernels of round r read round r-1's and the segmented kernel
// counts into the other one); launches are sized by the last count the host
// read, an upper bound since the count only shrinks.  The host reads the
// count back only every DR_SYNC rounds once fewer than DR_SYNC_MIN elements
// are active (and in rounds with groups above the shared-memory limit, whose
// side path is sized on the host), so small sorts run their rounds back to
// back; rounds launched after the count reached zero exit at once.  Large
// rounds read it every time: launches sized by a stale count cost more there
// (measured on the 512 MiB text: +0.3 ms with reads every 4th round only).
constexpr int DR_SYNC = 4;
constexpr uint32_t DR_SYNC_MIN = 1u << 20;
constexpr int DR_MAXR = 40;      // rounds recorded (h doubles each round: at most 33)
template <typename Rem>
static int doubling_rounds(Storage *st, uint32_t N, uint64_t h, uint32_t A, Rem rem, uint32_t *isa, uint32_t *sa,
                           uint32_t *act_x, uint32_t *act_g, uint32_t *act_x2, uint32_t *act_g2, bool check_big)
{
    static bool ss_attr = false;
    if (!ss_attr) {
        check_cuda(cudaFuncSetAttribute(k_seg_sort<Rem>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SS_SMEM));
        ss_attr = true;
    }
    const bool debug = getenv("GBWT_DEBUG") != nullptr;
    // device words: [0], [1] the two round counters, [2] the side path's
    // count, [8 + r] the active count round r started with
    uint32_t *dw = (uint32_t *)(st->d_scalars + 16);
    const uint32_t *hw = (const uint32_t *)(st->h_scalars + 160);   // pinned words past the byte tables
    check_cuda(cudaMemsetAsync(dw, 0, (8 + DR_MAXR) * 4, st->stream));
    k_set_word<<<1, 1, 0, st->stream>>>(dw + 1, A);     // round 0's count, read by round 1's kernels
    after_launch(st);
    uint32_t A_ub = A;
    bool exact = true;               // A_ub is the count itself, not a bound
    int r = 0;
    while (A_ub > 0) {
        if (r >= DR_MAXR) throw Error{GBWT_INTERNAL_ERROR};
        uint32_t *Aprev = dw + ((r + 1) & 1), *Acur = dw + (r & 1);
        if (h >= N) {
            // only legal when every suffix is finished already
            check_cuda(cudaMemcpyAsync(st->h_scalars + 160, dw, 8, cudaMemcpyDeviceToHost, st->stream));
            check_cuda(cudaStreamSynchronize(st->stream));
            if (hw[(r + 1) & 1] != 0) throw Error{GBWT_INTERNAL_ERROR};
            break;
        }
        const uint32_t h2 = (uint32_t)(2 * h < 0xFFFFFFFFull ? 2 * h : 0xFFFFFFFFull);
        // gather this round's keys before any rank changes; list big groups
        uint32_t *key2 = slot<uint32_t>(st, S_TMP2, N);
        const uint32_t ss_tiles = grid_for(A_ub, SS_TILE);
        uint32_t *tstart = slot<uint32_t>(st, S_SSTART, (size_t)ss_tiles * 2);
        uint32_t *tbig = tstart + ss_tiles;
        const uint32_t big_cap = A_ub / SS_SEGMAX + 1u;
        uint32_t *bigs = check_big ? slot<uint32_t>(st, S_BIGL, (size_t)big_cap * 2) : nullptr;
        if (check_big) check_cuda(cudaMemsetAsync(st->d_flags + 3, 0, 8, st->stream));
        check_cuda(cudaMemsetAsync(tstart, 0xFF, (size_t)ss_tiles * 4 * (check_big ? 2 : 1), st->stream));
        static_assert(SS_TILE % 256 == 0, "gather blocks must not straddle tiles");
        const uint32_t *Adev = exact ? nullptr : Aprev;     // a known count goes in as an argument
        k_round_gather<<<grid_for(A_ub, 256), 256, 0, st->stream>>>(act_x, act_g, isa, A_ub, Adev, (uint32_t)h,
                                                                    key2, st->d_flags, tstart, bigs, big_cap, tbig,
                                                                    dw + 8 + r);
        after_launch(st);
        uint32_t nbig = 0;
        if (check_big) {
            check_cuda(cudaMemcpyAsync(st->h_scalars + 2, st->d_flags + 3, 8, cudaMemcpyDeviceToHost, st->stream));
            check_cuda(cudaStreamSynchronize(st->stream));
            const uint32_t *cnt = (const uint32_t *)(st->h_scalars + 2);
            nbig = cnt[0];
            if (nbig > big_cap || cnt[1] != nbig) throw Error{GBWT_INTERNAL_ERROR};
        }
        check_big = nbig > 0;
        if (debug) fprintf(stderr, "gbwt: round h=%llu active<=%u big groups=%u\n", (unsigned long long)h, A_ub, nbig);
        check_cuda(cudaMemsetAsync(Acur, 0, 4, st->stream));
        if (debug) check_cuda(cudaMemsetAsync(st->d_flags + 16, 0, 8 * sizeof(uint32_t), st->stream));
        probe_begin(st, GBWT_PROBE_SEG_SORT);
        k_seg_sort<Rem><<<ss_tiles, SS_THREADS, SS_SMEM, st->stream>>>(
            act_x, act_g, key2, tstart, nbig ? tbig : nullptr, A_ub, Adev, h2, rem, isa, sa, act_x2, act_g2, Acur,
            st->d_flags, debug);
        // algorithmic bytes (24 per active element) are added once the
        // round's count is known, below
        probe_end(st, GBWT_PROBE_SEG_SORT, 0);
        after_launch(st);
        if (nbig) {
            big_groups<Rem>(st, N, nbig, bigs, big_cap, h2, key2, act_x, act_g, rem, isa, sa, act_x2, act_g2, Acur,
                            dw + 2);
            k_add_u32<<<1, 1, 0, st->stream>>>(Acur, dw + 2);
            after_launch(st);
        }
        uint32_t *t1 = act_x; act_x = act_x2; act_x2 = t1;
        uint32_t *t2 = act_g; act_g = act_g2; act_g2 = t2;
        h *= 2;
        r++;
        if (check_big || nbig || debug || A_ub >= DR_SYNC_MIN || r % DR_SYNC == 0) {
            check_cuda(cudaMemcpyAsync(st->h_scalars + 160, dw, 8, cudaMemcpyDeviceToHost, st->stream));
            check_cuda(cudaStreamSynchronize(st->stream));
            A_ub = hw[(r + 1) & 1];        // the count this round produced (r already advanced)
            exact = true;
            if (debug) {
                uint32_t tiers[8];
                check_cuda(cudaMemcpy(tiers, st->d_flags + 16, sizeof(tiers), cudaMemcpyDeviceToHost));
                fprintf(stderr, "gbwt:   groups=%u elements in groups <=%u: %u, <=%u: %u, larger: %u\n", tiers[3],
                        SS_COUNTMAX, tiers[0], SS_WARPMAX, tiers[1], tiers[2]);
                fprintf(stderr, "gbwt:   larger groups: one value %u, majority + <=32 outliers %u, other %u\n",
                        tiers[4], tiers[7], tiers[6]);
            }
        } else {
            exact = false;
        }
    }
    // rounds that had work, and the probe's algorithmic bytes per round
    check_cuda(cudaMemcpyAsync(st->h_scalars + 160, dw, (8 + DR_MAXR) * 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    int rounds = 0;
    for (int i = 0; i < r; i++) {
        const uint32_t a = hw[8 + i];
        if (a == 0) break;
        rounds++;
        if (st->probe_kernel == GBWT_PROBE_SEG_SORT) st->probe_bytes += (int64_t)24 * a;
    }
    // launches of rounds that found nothing to do are not counted
    if (st->probe_kernel == GBWT_PROBE_SEG_SORT) st->probe_launches -= r - rounds;
    return rounds;
}

// Sorts N positions; key0 (in slot S_KEY0) holds the initial keys covering
// h0 symbols; with key0_cont, bit 0 of every initial key tells whether the
// suffix is longer than h0 (rem > h0).  Fills isa[N] and sa[N]; returns the
// number of rounds.
template <typename Rem>
static int prefix_doubling(Storage *st, uint32_t N, int key0_bits, uint32_t h0, Rem rem, uint32_t *isa,
                           uint32_t *sa, bool key0_cont = false)
{
    uint64_t *keys = slot<uint64_t>(st, S_KEY0, N);
    uint64_t *keys_alt = slot<uint64_t>(st, S_KEY1, N);
    uint32_t *vals = slot<uint32_t>(st, S_VAL0, N);
    uint32_t *vals_alt = slot<uint32_t>(st, S_VAL1, N);
    uint32_t *act_x = slot<uint32_t>(st, S_ACTX, N);
    uint32_t *act_g = slot<uint32_t>(st, S_ACTG, N);
    uint32_t *act_x2 = slot<uint32_t>(st, S_ACTX2, N);   // next active list
    uint32_t *act_g2 = slot<uint32_t>(st, S_ACTG2, N);

    k_iota<<<grid_for(N, 256), 256, 0, st->stream>>>(vals, N);
    after_launch(st);
    radix_sort<uint64_t, true>(st, keys, keys_alt, vals, vals_alt, N, 0, key0_bits);
    ActiveTest<Rem> at{keys, vals, N, h0, rem};
    check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
    device_scan<uint64_t, OpMaxAdd>(st, N, LoadHeadActive0<Rem>{at, key0_cont},
                                    StoreHeadActive0<Rem>{at, isa, sa, act_x, act_g},
                                    false, (uint64_t *)st->d_scalars);
    fetch_scalars(st, 1);
    const uint32_t A = (uint32_t)st->h_scalars[0];      // low word of the total: active elements
    return 1 + doubling_rounds(st, N, h0, A, rem, isa, sa, act_x, act_g, act_x2, act_g2, true);
}

// Byte values present in the dictionary (= the text's alphabet plus the
// sentinel byte 1), as a 256-bit set OR-ed into bits[0..8).
__global__ void k_alpha_present(const uint8_t *dict, uint32_t N, uint32_t *bits)
{
    uint32_t m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t x = blockIdx.x * blockDim.x + threadIdx.x; x < N; x += gridDim.x * blockDim.x) {
        const uint32_t c = dict[x];
#pragma unroll
        for (int w = 0; w < 8; w++) m[w] |= ((c >> 5) == (uint32_t)w) ? (1u << (c & 31u)) : 0u;
    }
#pragma unroll
    for (int w = 0; w < 8; w++) {
        const uint32_t v = __reduce_or_sync(0xFFFFFFFFu, m[w]);
        if ((threadIdx.x & 31u) == 0 && v) atomicOr(bits + w, v);
    }
}

// Initial dictionary keys: the next h0 symbols of the phrase suffix, each
// recoded to its rank in the alphabet (code 0 = past the phrase end, `bps`
// bits per symbol, h0 = floor(63 / bps): 21 symbols for DNA, 7 for a full
// byte alphabet), then one bit "the suffix continues past h0".  The bit keeps
// every group uniform in whether its strings end within h0 symbols: without
// it a suffix of exactly h0 symbols would tie with longer suffixes sharing
// those symbols.  The recoding is monotone, so the order is the byte order.
// Also writes rem8[x] = min(rem(x), 255) (see DictRem).
__global__ void k_dict_keys(const uint8_t *dict, uint32_t N, DictRem rem, const uint8_t *code, int bps, int h0,
                            uint64_t *keys, uint8_t *rem8)
{
    __shared__ uint8_t s_code[256];
    s_code[threadIdx.x] = code[threadIdx.x];     // blockDim == 256
    __syncthreads();
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= N) return;
    const uint32_t r = rem(x);
    uint64_t key = 0;
    for (int i = 0; i < h0; i++) key = (key << bps) | (uint64_t)((uint32_t)i < r ? s_code[dict[x + i]] : 0u);
    key = (key << 1) | (r > (uint32_t)h0 ? 1u : 0u);
    keys[x] = key;
    rem8[x] = (uint8_t)(r < 255u ? r : 255u);
}

// Dense lexicographic rank of each distinct phrase.  After the sort, isa[x]
// is the head of x's group in sa; distinct phrases never share a group, so
// the phrase starts' heads are distinct and their order is the phrases'
// order.  The heads are marked in a bit vector over sa positions; a phrase's
// rank is the number of marks before its head (word popcount prefix plus the
// popcount inside the word).  That touches d phrases and N/32 words instead
// of all N dictionary positions.
__global__ void k_mark_phrase_heads(const uint32_t *isa, const uint32_t *doff, uint32_t d, uint32_t *bits)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d) return;
    const uint32_t p = isa[doff[q]];
    atomicOr(&bits[p >> 5], 1u << (p & 31));
}
struct LoadPopc {
    const uint32_t *bits;
    __device__ __forceinline__ uint32_t operator()(size_t t) const { return (uint32_t)__popc(bits[t]); }
};
struct StoreWordPre {
    uint32_t *pre;
    __device__ __forceinline__ void operator()(size_t t, uint32_t p, uint32_t) const { pre[t] = p; }
};
__global__ void k_phrase_lexrank(const uint32_t *isa, const uint32_t *doff, uint32_t d, const uint32_t *bits,
                                 const uint32_t *pre, uint32_t *lexrank)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d) return;
    const uint32_t p = isa[doff[q]];
    const uint32_t w = p >> 5;
    lexrank[q] = pre[w] + (uint32_t)__popc(bits[w] & ((1u << (p & 31)) - 1u));
}

void run_dict_sort(Storage *st, Phrases &ph, int W, bool small, DictOrder &dord)
{
    (void)W;
    (void)small;   // the alphabet recoding below covers the small-alphabet packing
    const uint32_t N = (uint32_t)ph.dict_bytes;
    DictRem rem{ph.dphr, ph.doff, ph.dlen, nullptr};
    // alphabet of the dictionary -> dense codes 1..sigma
    check_cuda(cudaMemsetAsync(st->d_flags + 8, 0, 8 * sizeof(uint32_t), st->stream));
    unsigned ag = grid_for(N, 256);
    if (ag > (unsigned)st->num_sms * 4) ag = (unsigned)st->num_sms * 4;
    k_alpha_present<<<ag, 256, 0, st->stream>>>(ph.dict, N, st->d_flags + 8);
    after_launch(st);
    uint32_t present[8];
    check_cuda(cudaMemcpyAsync(st->h_scalars + 4, st->d_flags + 8, sizeof(present), cudaMemcpyDeviceToHost,
                               st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    memcpy(present, st->h_scalars + 4, sizeof(present));
    uint8_t *hcode = (uint8_t *)(st->h_scalars + 16);          // 256 pinned bytes
    uint32_t sigma = 0;
    for (int c = 0; c < 256; c++) {
        const bool p = (present[c >> 5] >> (c & 31)) & 1u;
        hcode[c] = p ? (uint8_t)(++sigma) : 0;
    }
    const int bps = bits_for(sigma);                           // codes 0..sigma
    // as many symbols as fit the first key's bit budget (radix passes over
    // the dictionary vs later doubling rounds: a tuning knob)
    const int key_bits = tune_dict_key_bits(st);
    const int h0 = (key_bits - 1) / bps > 0 ? (key_bits - 1) / bps : 1;
    uint8_t *dcode = slot<uint8_t>(st, S_TMP1, 256);
    check_cuda(cudaMemcpyAsync(dcode, hcode, 256, cudaMemcpyHostToDevice, st->stream));
    uint64_t *keys = slot<uint64_t>(st, S_KEY0, N);
    uint8_t *rem8 = slot<uint8_t>(st, S_TMP0, N);
    k_dict_keys<<<grid_for(N, 256), 256, 0, st->stream>>>(ph.dict, N, rem, dcode, bps, h0, keys, rem8);
    after_launch(st);
    rem.rem8 = rem8;
    dord.isa = slot<uint32_t>(st, S_ISA, N);
    dord.sa = slot<uint32_t>(st, S_SA, N);
    dord.rounds = prefix_doubling(st, N, h0 * bps + 1, (uint32_t)h0, rem, dord.isa, dord.sa, true);
    dord.lexrank = slot<uint32_t>(st, S_LEXRANK, ph.d);
    const size_t words = ((size_t)N + 31) / 32;
    uint32_t *bits = slot<uint32_t>(st, S_TMP0, words);
    uint32_t *pre = slot<uint32_t>(st, S_TMP2, words);
    check_cuda(cudaMemsetAsync(bits, 0, words * sizeof(uint32_t), st->stream));
    k_mark_phrase_heads<<<grid_for(ph.d, 256), 256, 0, st->stream>>>(dord.isa, ph.doff, ph.d, bits);
    after_launch(st);
    device_scan<uint32_t, OpAdd>(st, words, LoadPopc{bits}, StoreWordPre{pre}, false, (uint32_t *)nullptr);
    k_phrase_lexrank<<<grid_for(ph.d, 256), 256, 0, st->stream>>>(dord.isa, ph.doff, ph.d, bits, pre,
                                                                   dord.lexrank);
    after_launch(st);
}

// First parse key: one phrase rank (two == false), or two (the second 0
// past the parse end).
__global__ void k_parse_keys(const uint32_t *pid, const uint32_t *lexrank, uint32_t z, int lb, bool two,
                             uint64_t *keys)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= z) return;
    uint64_t a = lexrank[pid[i]];
    if (!two) { keys[i] = a; return; }
    uint64_t b = i + 1 < z ? (uint64_t)lexrank[pid[i + 1]] + 1u : 0u;
    keys[i] = (a << lb) | b;
}

// Parse round 0 without a sort.  The parse suffix array lists the
// occurrences of each phrase contiguously, phrases in lexicographic order, so
// the first-round group of an occurrence is its phrase's bucket, which starts
// at the number of occurrences of all lower-ranked phrases.  Every
// occurrence's rank is written in place (coalesced); occurrences of phrases
// that occur once are finished; the others go to the active list bucket by
// bucket, in no particular order inside a bucket: the rounds sort every
// group by its next key and all parse suffixes differ, so no order among
// equal keys survives to the result.
__global__ void k_bucket_counts(const uint32_t *lexrank, const uint32_t *occ, uint32_t d, uint32_t *cnt_r)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q < d) cnt_r[lexrank[q]] = occ[q];
}
// packed per rank: (occurrences << 32) | (occurrences staying active)
struct LoadBucket {
    const uint32_t *cnt;
    __device__ __forceinline__ uint64_t operator()(size_t r) const
    {
        const uint32_t c = cnt[r];
        return ((uint64_t)c << 32) | (c > 1u ? c : 0u);
    }
};
struct StoreBucket {
    uint64_t *bst;
    __device__ __forceinline__ void operator()(size_t r, uint64_t pre, uint64_t) const { bst[r] = pre; }
};
// Per phrase: (bucket start, active-list start), the second 0xFFFFFFFF for a
// phrase that occurs once.  One random lookup per occurrence instead of three
// (rank, bucket, count) in the scatter below.
__global__ void k_bucket_info(const uint32_t *lexrank, const uint64_t *bst, const uint32_t *occ, uint32_t d,
                              uint2 *info)
{
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= d) return;
    const uint64_t p = bst[lexrank[q]];
    info[q] = make_uint2((uint32_t)(p >> 32), occ[q] > 1u ? (uint32_t)p : 0xFFFFFFFFu);
}
__global__ void k_bucket_scatter(const uint32_t *pid, const uint2 *info, uint32_t z, uint32_t *cur, uint32_t *isa,
                                 uint32_t *sa, uint32_t *act_x, uint32_t *act_g, uint32_t *flags)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= z) return;
    const uint32_t q = pid[i];
    const uint2 inf = info[q];
    const uint32_t b = inf.x;
    isa[i] = b;
    if (inf.y == 0xFFFFFFFFu) {
        if (b < z) sa[b] = i;         // the only suffix starting with this phrase
        else atomicOr(flags, ERR_INTERNAL);
    } else {
        const uint32_t pos = inf.y + atomicAdd(cur + q, 1u);
        if (pos < z) {
            act_x[pos] = i;
            act_g[pos] = b;
        } else {
            atomicOr(flags, ERR_INTERNAL);
        }
    }
}

void run_parse_sa(Storage *st, Phrases &ph, DictOrder &dord, ParseOrder &pord)
{
    const uint32_t z = ph.z;
    pord.isa = slot<uint32_t>(st, S_PISA, z);
    pord.sa = slot<uint32_t>(st, S_PSA, z);
    const int kp = tune_parse_key_phrases(st);
    if (kp == 1 || kp == 2) {
        // round 0 by a radix sort of the first one or two phrase ranks
        uint64_t *keys = slot<uint64_t>(st, S_KEY0, z);
        const int lb = bits_for(ph.d);       // lexrank+1 <= d
        k_parse_keys<<<grid_for(z, 256), 256, 0, st->stream>>>(ph.pid, dord.lexrank, z, lb, kp == 2, keys);
        after_launch(st);
        pord.rounds = prefix_doubling(st, z, kp == 2 ? lb + bits_for(ph.d - 1) : bits_for(ph.d - 1), (uint32_t)kp,
                                      ParseRem{z}, pord.isa, pord.sa);
        return;
    }
    // round 0 from the phrase buckets (the last phrase occurs once: its
    // suffix, the only one ending within one phrase, is finished here)
    const uint32_t d = ph.d;
    uint32_t *cnt_r = slot<uint32_t>(st, S_TMP0, d);
    uint64_t *bst = slot<uint64_t>(st, S_KEY1, d);
    uint32_t *cur = slot<uint32_t>(st, S_TMP1, d);
    uint32_t *act_x = slot<uint32_t>(st, S_ACTX, z);
    uint32_t *act_g = slot<uint32_t>(st, S_ACTG, z);
    uint32_t *act_x2 = slot<uint32_t>(st, S_ACTX2, z);
    uint32_t *act_g2 = slot<uint32_t>(st, S_ACTG2, z);
    k_bucket_counts<<<grid_for(d, 256), 256, 0, st->stream>>>(dord.lexrank, ph.occ, d, cnt_r);
    after_launch(st);
    check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
    device_scan<uint64_t, OpAdd>(st, d, LoadBucket{cnt_r}, StoreBucket{bst}, false, (uint64_t *)st->d_scalars);
    check_cuda(cudaMemsetAsync(cur, 0, (size_t)d * 4, st->stream));
    uint2 *info = slot<uint2>(st, S_KEY0, d);
    k_bucket_info<<<grid_for(d, 256), 256, 0, st->stream>>>(dord.lexrank, bst, ph.occ, d, info);
    after_launch(st);
    k_bucket_scatter<<<grid_for(z, 256), 256, 0, st->stream>>>(ph.pid, info, z, cur, pord.isa, pord.sa, act_x, act_g,
                                                               st->d_flags);
    after_launch(st);
    fetch_scalars(st, 1);
    const uint64_t tot = st->h_scalars[0];
    if ((uint32_t)(tot >> 32) != z) throw Error{GBWT_INTERNAL_ERROR};
    pord.rounds = 1 + doubling_rounds(st, z, 1, (uint32_t)tot, ParseRem{z}, pord.isa, pord.sa, act_x, act_g, act_x2,
                                      act_g2, true);
}

// Batch: the second symbol of a key is 0 when phrase i ends its text.
__global__ void k_parse_keys_batch(const uint32_t *pid, const uint32_t *lexrank, const uint32_t *ptid, uint32_t z,
                                   int lb, bool two, uint64_t *keys)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= z) return;
    uint64_t a = lexrank[pid[i]];
    if (!two) { keys[i] = a; return; }
    uint64_t b = (i + 1 < z && ptid[i + 1] == ptid[i]) ? (uint64_t)lexrank[pid[i + 1]] + 1u : 0u;
    keys[i] = (a << lb) | b;
}

// Suffix array over all texts' parses at once.  Suffixes of different texts
// may be equal strings and then share a rank; the order restricted to one
// text is that text's own parse suffix array.
void run_parse_sa_batch(Storage *st, Phrases &ph, DictOrder &dord, const BatchText &bt, ParseOrder &pord)
{
    const uint32_t z = ph.z;
    uint64_t *keys = slot<uint64_t>(st, S_KEY0, z);
    const int lb = bits_for(ph.d);
    const bool two = tune_parse_key_phrases(st) != 1;
    k_parse_keys_batch<<<grid_for(z, 256), 256, 0, st->stream>>>(ph.pid, dord.lexrank, bt.ptid, z, lb, two, keys);
    after_launch(st);
    uint32_t *remv = slot<uint32_t>(st, S_TMP0, z);
    k_batch_rem<<<grid_for(z, 256), 256, 0, st->stream>>>(bt.ptid, bt.zend, z, remv);
    after_launch(st);
    // bitmap words for positions up to z + BR_MAPH (ranges reach past z)
    const size_t map_words = ((size_t)z + BR_MAPH + 64u * 32u) / (64u * 32u) + 1u;
    uint32_t *endmap = slot<uint32_t>(st, S_TMP1, map_words);
    check_cuda(cudaMemsetAsync(endmap, 0, map_words * 4, st->stream));
    k_text_endmap<<<grid_for(bt.k, 256), 256, 0, st->stream>>>(bt.zend, bt.k, endmap);
    after_launch(st);
    pord.isa = slot<uint32_t>(st, S_PISA, z);
    pord.sa = slot<uint32_t>(st, S_PSA, z);
    pord.rounds = prefix_doubling(st, z, two ? lb + bits_for(ph.d - 1) : bits_for(ph.d - 1), two ? 2u : 1u,
                                  BatchParseRem{remv, endmap}, pord.isa, pord.sa);
}

}  // namespace gbwt
