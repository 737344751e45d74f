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
// keyed on isa[x+h] inherits it from the groups of x+h.  Keys are (group, isa[x+h]+1)
// sorted with the project's stable LSD radix sort; group starts and new heads
// come from one component-wise max-scan.
#include "prims.cuh"

namespace gbwt {

struct DictRem {
    const uint32_t *dphr, *doff, *dlen;
    __device__ __forceinline__ uint32_t operator()(uint32_t x) const
    {
        uint32_t q = dphr[x];
        return doff[q] + dlen[q] - x;
    }
};
struct ParseRem {
    uint32_t n;
    __device__ __forceinline__ uint32_t operator()(uint32_t x) const { return n - x; }
};

__global__ void k_iota(uint32_t *v, uint32_t n)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] = i;
}

// Round 0 heads: max-scan of (new key ? t : 0).
struct LoadKeyHead {
    const uint64_t *k;
    __device__ __forceinline__ uint32_t operator()(size_t t) const
    {
        return (t == 0 || k[t] != k[t - 1]) ? (uint32_t)t : 0u;
    }
};
struct StoreHead0 {
    const uint32_t *vals;
    uint32_t *isa;
    uint32_t *head;
    __device__ __forceinline__ void operator()(size_t t, uint32_t h, uint32_t) const
    {
        isa[vals[t]] = h;
        head[t] = h;
    }
};

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
        return single || rem(vals[t]) <= h;
    }
};

template <typename Rem>
struct LoadActive {
    ActiveTest<Rem> a;
    __device__ __forceinline__ uint32_t operator()(size_t t) const { return a.done(t) ? 0u : 1u; }
};
// Compaction of the active elements; finished ones are written to sa[].
// `pos` gives an element's final position (round 0: t; later rounds: from
// the head array, see StoreRound).
template <typename Rem>
struct StoreActive0 {
    ActiveTest<Rem> a;
    const uint32_t *head;
    uint32_t *sa;
    uint32_t *act_x;
    uint32_t *act_g;
    __device__ __forceinline__ void operator()(size_t t, uint32_t pre, uint32_t v) const
    {
        const uint32_t x = a.vals[t];
        if (v) {
            act_x[pre] = x;
            act_g[pre] = head[t];
        } else {
            sa[t] = x;
        }
    }
};

// Round keys: (group head, isa[x+h] + 1).
__global__ void k_round_keys(const uint32_t *act_x, const uint32_t *act_g, const uint32_t *isa, uint32_t A,
                             uint32_t h, int lb, uint64_t *keys, uint32_t *vals)
{
    uint32_t a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A) return;
    const uint32_t x = act_x[a];
    keys[a] = ((uint64_t)act_g[a] << lb) | (uint64_t)(isa[x + h] + 1u);
    vals[a] = x;
}

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
template <typename Rem>
struct StoreRound {
    ActiveTest<Rem> t;
    int lb;
    uint32_t *isa;
    uint32_t *head;
    uint32_t *sa;
    __device__ __forceinline__ void operator()(size_t a, uint64_t inc, uint64_t) const
    {
        const uint32_t g = (uint32_t)(t.k[a] >> lb);
        const uint32_t ag = (uint32_t)(inc >> 32), s2 = (uint32_t)inc;
        const uint32_t nh = g + (s2 - ag);
        const uint32_t x = t.vals[a];
        isa[x] = nh;
        head[a] = nh;
        if (t.done(a)) sa[g + ((uint32_t)a - ag)] = x;
    }
};
template <typename Rem>
struct StoreActiveR {
    ActiveTest<Rem> a;
    const uint32_t *head;
    uint32_t *act_x;
    uint32_t *act_g;
    __device__ __forceinline__ void operator()(size_t t, uint32_t pre, uint32_t v) const
    {
        if (v) {
            act_x[pre] = a.vals[t];
            act_g[pre] = head[t];
        }
    }
};

// Sorts N positions; key0 (in slot S_KEY0) holds the initial keys covering
// h0 symbols.  Fills isa[N] and sa[N]; returns the number of rounds.
template <typename Rem>
static int prefix_doubling(Storage *st, uint32_t N, int key0_bits, uint32_t h0, Rem rem, uint32_t *isa,
                           uint32_t *sa)
{
    uint64_t *keys = slot<uint64_t>(st, S_KEY0, N);
    uint64_t *keys_alt = slot<uint64_t>(st, S_KEY1, N);
    uint32_t *vals = slot<uint32_t>(st, S_VAL0, N);
    uint32_t *vals_alt = slot<uint32_t>(st, S_VAL1, N);
    uint32_t *act_x = slot<uint32_t>(st, S_ACTX, N);
    uint32_t *act_g = slot<uint32_t>(st, S_ACTG, N);
    uint32_t *head = slot<uint32_t>(st, S_HEAD, N);
    int rounds = 1;

    k_iota<<<grid_for(N, 256), 256, 0, st->stream>>>(vals, N);
    after_launch(st);
    radix_sort<uint64_t, true>(st, keys, keys_alt, vals, vals_alt, N, 0, key0_bits);
    device_scan<uint32_t, OpMax>(st, N, LoadKeyHead{keys}, StoreHead0{vals, isa, head}, true, (uint32_t *)nullptr);
    ActiveTest<Rem> at{keys, vals, N, h0, rem};
    check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
    device_scan<uint32_t, OpAdd>(st, N, LoadActive<Rem>{at}, StoreActive0<Rem>{at, head, sa, act_x, act_g}, false,
                                 (uint32_t *)st->d_scalars);
    fetch_scalars(st, 1);
    uint32_t A = (uint32_t)st->h_scalars[0];
    const int lb = bits_for(N);          // isa+1 <= N
    const int gb = bits_for(N - 1);
    uint64_t h = h0;
    while (A > 0) {
        if (h >= N) throw Error{GBWT_INTERNAL_ERROR};
        // the key arrays of the previous round are dead: rebuild in place
        uint64_t *k = slot<uint64_t>(st, S_KEY0, N);
        uint64_t *k_alt = slot<uint64_t>(st, S_KEY1, N);
        uint32_t *v = slot<uint32_t>(st, S_VAL0, N);
        uint32_t *v_alt = slot<uint32_t>(st, S_VAL1, N);
        k_round_keys<<<grid_for(A, 256), 256, 0, st->stream>>>(act_x, act_g, isa, A, (uint32_t)h, lb, k, v);
        after_launch(st);
        radix_sort<uint64_t, true>(st, k, k_alt, v, v_alt, A, 0, lb + gb);
        ActiveTest<Rem> t{k, v, A, (uint32_t)(2 * h < 0xFFFFFFFFull ? 2 * h : 0xFFFFFFFFull), rem};
        device_scan<uint64_t, OpMax2>(st, A, LoadRoundHead{k, lb}, StoreRound<Rem>{t, lb, isa, head, sa}, true,
                                      (uint64_t *)nullptr);
        check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
        device_scan<uint32_t, OpAdd>(st, A, LoadActive<Rem>{t}, StoreActiveR<Rem>{t, head, act_x, act_g}, false,
                                     (uint32_t *)st->d_scalars);
        fetch_scalars(st, 1);
        A = (uint32_t)st->h_scalars[0];
        h *= 2;
        rounds++;
    }
    return rounds;
}

// Initial dictionary keys: the next h0 = 7 bytes (or 15 four-bit symbols with
// the small alphabet) of the phrase suffix, zero past the phrase end, then one
// bit "the suffix continues past h0".  The bit keeps every group uniform in
// whether its strings end within h0 symbols: without it a suffix of exactly
// h0 symbols would tie with longer suffixes sharing those symbols.
constexpr uint32_t DICT_H0 = 7, DICT_H0_SMALL = 15;

__global__ void k_dict_keys(const uint8_t *dict, uint32_t N, DictRem rem, bool small, uint64_t *keys)
{
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= N) return;
    const uint32_t r = rem(x);
    uint64_t key = 0;
    if (small) {
#pragma unroll
        for (int i = 0; i < (int)DICT_H0_SMALL; i++)
            key = (key << 4) | (uint64_t)((uint32_t)i < r ? (dict[x + i] & 15u) : 0u);
        key = (key << 1) | (r > DICT_H0_SMALL ? 1u : 0u);
    } else {
#pragma unroll
        for (int i = 0; i < (int)DICT_H0; i++) key = (key << 8) | (uint64_t)((uint32_t)i < r ? dict[x + i] : 0u);
        key = (key << 1) | (r > DICT_H0 ? 1u : 0u);
    }
    keys[x] = key;
}

// Dense lexicographic rank of each distinct phrase (positions at offset 0).
struct LoadIsStart {
    const uint32_t *sa;
    const uint32_t *dphr, *doff;
    __device__ __forceinline__ uint32_t operator()(size_t t) const
    {
        uint32_t x = sa[t];
        return doff[dphr[x]] == x ? 1u : 0u;
    }
};
struct StoreLexRank {
    const uint32_t *sa;
    const uint32_t *dphr;
    uint32_t *lexrank;
    __device__ __forceinline__ void operator()(size_t t, uint32_t pre, uint32_t v) const
    {
        if (v) lexrank[dphr[sa[t]]] = pre;
    }
};

void run_dict_sort(Storage *st, Phrases &ph, int W, bool small, DictOrder &dord)
{
    (void)W;
    const uint32_t N = (uint32_t)ph.dict_bytes;
    DictRem rem{ph.dphr, ph.doff, ph.dlen};
    uint64_t *keys = slot<uint64_t>(st, S_KEY0, N);
    k_dict_keys<<<grid_for(N, 256), 256, 0, st->stream>>>(ph.dict, N, rem, small, keys);
    after_launch(st);
    dord.isa = slot<uint32_t>(st, S_ISA, N);
    dord.sa = slot<uint32_t>(st, S_SA, N);
    dord.rounds = prefix_doubling(st, N, small ? 61 : 57, small ? DICT_H0_SMALL : DICT_H0, rem, dord.isa, dord.sa);
    dord.lexrank = slot<uint32_t>(st, S_LEXRANK, ph.d);
    device_scan<uint32_t, OpAdd>(st, N, LoadIsStart{dord.sa, ph.dphr, ph.doff},
                                 StoreLexRank{dord.sa, ph.dphr, dord.lexrank}, false, (uint32_t *)nullptr);
}

__global__ void k_parse_keys(const uint32_t *pid, const uint32_t *lexrank, uint32_t z, int lb, uint64_t *keys)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= z) return;
    uint64_t a = lexrank[pid[i]];
    uint64_t b = i + 1 < z ? (uint64_t)lexrank[pid[i + 1]] + 1u : 0u;
    keys[i] = (a << lb) | b;
}

void run_parse_sa(Storage *st, Phrases &ph, DictOrder &dord, ParseOrder &pord)
{
    const uint32_t z = ph.z;
    uint64_t *keys = slot<uint64_t>(st, S_KEY0, z);
    const int lb = bits_for(ph.d);       // lexrank+1 <= d
    k_parse_keys<<<grid_for(z, 256), 256, 0, st->stream>>>(ph.pid, dord.lexrank, z, lb, keys);
    after_launch(st);
    pord.isa = slot<uint32_t>(st, S_PISA, z);
    pord.sa = slot<uint32_t>(st, S_PSA, z);
    pord.rounds = prefix_doubling(st, z, lb + bits_for(ph.d - 1), 2u, ParseRem{z}, pord.isa, pord.sa);
}

}  // namespace gbwt
