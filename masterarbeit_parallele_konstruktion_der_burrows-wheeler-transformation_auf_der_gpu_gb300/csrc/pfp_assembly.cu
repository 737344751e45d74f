// pfp_assembly.cu -- BWT assembly from the dictionary order and the parse
// suffix array (sm_103a).
//
// The reference enumerates S (distinct phrase suffixes longer than W) from a
// colex sort of all occurrences, finds each entry's colex interval with a
// next-smaller-value search, writes one-byte blocks ("runs") directly and
// sorts the remaining ("mixed") blocks by the rank of the next parse suffix
// (Prefix_Free_Parsing_W=5_P=16_kommentiert.cu, "K": Compute_S1..S6
// K:2509-3369, bitonic block sorts K:3556-4248).
//
// Here S comes out of the dictionary suffix order directly: equal suffixes
// are one group of the prefix-doubling result.  For every group we add the
// occurrence counts of its phrases (block length) and check whether all
// preceding bytes agree (run).  Runs are written one group per thread with
// 16-byte stores (long blocks one CTA each).  For mixed groups, every phrase
// occurrence -- visited in parse
// suffix-array order, which is exactly the "rank of the next parse suffix"
// order the reference sorts by -- emits one (group, byte) element per mixed
// suffix of its phrase; one stable radix sort by group then places every
// byte, and a coalesced scatter writes them into the output.
#include "prims.cuh"

namespace gbwt {

constexpr uint32_t PC_VAR = 0x100u;     // "byte preceding the occurrence"

struct PosInfo {
    const uint32_t *dphr, *doff, *dlen;
    __device__ __forceinline__ void get(uint32_t x, uint32_t &q, uint32_t &off, uint32_t &rem) const
    {
        q = dphr[x];
        off = x - doff[q];
        rem = dlen[q] - off;
    }
};

// Preceding-byte code of the phrase suffix starting at dictionary position x.
__device__ __forceinline__ uint32_t pc_code(const uint8_t *dict, const uint32_t *pcmin, const uint32_t *pcmax,
                                            uint32_t x, uint32_t q, uint32_t off)
{
    if (off) return dict[x - 1];
    return pcmin[q] == pcmax[q] ? pcmin[q] : PC_VAR;
}

// S groups (equal phrase suffixes longer than W) in dictionary order.  The
// passes run over dictionary positions x in storage order, so the phrase
// tables are read almost sequentially: (1) mark the sorted position isa[x]
// of every long suffix's group head, (2) scan the marks into group numbers,
// (3) read each position's group back through isa[x].
__global__ void k_mark_sheads(uint32_t N, PosInfo pi, uint32_t W, const uint32_t *isa, uint8_t *mark)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= N) return;
    uint32_t q, off, rem;
    pi.get(x, q, off, rem);
    if (rem > W) mark[isa[x]] = 1;
}
struct LoadMark {
    const uint8_t *m;
    __device__ __forceinline__ uint32_t operator()(size_t t) const { return m[t]; }
};
struct StoreGid {
    const uint8_t *m;
    uint32_t *gid;
    __device__ __forceinline__ void operator()(size_t t, uint32_t inc, uint32_t v) const
    {
        if (v) gid[t] = inc - 1u;
    }
};

// Group of every long suffix; with `gcount` also the block lengths (sum of
// the phrases' occurrence counts) and one preceding-byte code per group
// (any member's: the mixed test compares every member with it).
__global__ void k_group_of(uint32_t N, PosInfo pi, uint32_t W, const uint32_t *isa, const uint32_t *gid,
                           uint32_t *grp_of, const uint8_t *dict, const uint32_t *occ, const uint32_t *pcmin,
                           const uint32_t *pcmax, uint32_t *gcount, uint16_t *gchar)
{
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= N) return;
    uint32_t q, off, rem;
    pi.get(x, q, off, rem);
    if (rem <= W) return;
    const uint32_t g = gid[isa[x]];
    grp_of[x] = g;
    if (gcount) {
        atomicAdd(gcount + g, occ[q]);
        gchar[g] = (uint16_t)pc_code(dict, pcmin, pcmax, x, q, off);
    }
}

// Passes (1)-(2); returns the number of groups, gid in slot S_TMP0.
static uint32_t group_numbers(Storage *st, Phrases &ph, DictOrder &dord, int W, uint32_t *&gid)
{
    const uint32_t N = (uint32_t)ph.dict_bytes;
    PosInfo pi{ph.dphr, ph.doff, ph.dlen};
    uint8_t *mark = slot<uint8_t>(st, S_MB, N);
    gid = slot<uint32_t>(st, S_TMP0, N);
    check_cuda(cudaMemsetAsync(mark, 0, N, st->stream));
    k_mark_sheads<<<grid_for(N, 256), 256, 0, st->stream>>>(N, pi, (uint32_t)W, dord.isa, mark);
    after_launch(st);
    check_cuda(cudaMemsetAsync(st->d_scalars, 0, 8, st->stream));
    device_scan<uint32_t, OpAdd>(st, N, LoadMark{mark}, StoreGid{mark, gid}, true, (uint32_t *)st->d_scalars);
    fetch_scalars(st, 1);
    return (uint32_t)st->h_scalars[0];
}

// Pass 2 over dictionary positions: mark groups with differing bytes.
__global__ void k_mark_mixed(uint32_t N, PosInfo pi, uint32_t W, const uint8_t *dict, const uint32_t *pcmin,
                             const uint32_t *pcmax, const uint32_t *grp_of, const uint16_t *gchar, uint8_t *gmix)
{
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= N) return;
    uint32_t q, off, rem;
    pi.get(x, q, off, rem);
    if (rem <= W) return;
    const uint32_t g = grp_of[x];
    const uint32_t c = pc_code(dict, pcmin, pcmax, x, q, off);
    if (c == PC_VAR || c != gchar[g]) gmix[g] = 1;
}

struct LoadGCount {
    const uint32_t *gcount;
    __device__ __forceinline__ uint32_t operator()(size_t g) const { return gcount[g]; }
};
// Mixed groups: packed (count of mixed groups, bytes in mixed groups).
struct LoadMixPair {
    const uint32_t *gcount;
    const uint8_t *gmix;
    __device__ __forceinline__ uint64_t operator()(size_t g) const
    {
        return gmix[g] ? ((1ull << 32) | gcount[g]) : 0ull;
    }
};
struct StoreMix {
    const uint8_t *gmix;
    const uint32_t *goff;
    uint32_t *mixidx;
    uint32_t *delta;
    __device__ __forceinline__ void operator()(size_t g, uint64_t pre, uint64_t) const
    {
        if (!gmix[g]) return;
        const uint32_t b = (uint32_t)(pre >> 32), mstart = (uint32_t)pre;
        mixidx[g] = b;
        delta[b] = goff[g] - mstart;
    }
};

// Per-phrase lists of mixed suffixes, in dictionary (phrase, offset) order.
struct LoadMixEntry {
    PosInfo pi;
    uint32_t W;
    const uint32_t *grp_of;
    const uint8_t *gmix;
    __device__ __forceinline__ uint32_t operator()(size_t x) const
    {
        uint32_t q, off, rem;
        pi.get((uint32_t)x, q, off, rem);
        return (rem > W && gmix[grp_of[x]]) ? 1u : 0u;
    }
};
struct StoreMixEntry {
    PosInfo pi;
    const uint8_t *dict;
    const uint32_t *grp_of, *mixidx;
    uint32_t *moff;
    uint32_t *mb;
    uint16_t *mc;
    __device__ __forceinline__ void operator()(size_t x, uint32_t pre, uint32_t v) const
    {
        uint32_t q, off, rem;
        pi.get((uint32_t)x, q, off, rem);
        if (off == 0) moff[q] = pre;
        if (v) {
            mb[pre] = mixidx[grp_of[x]];
            mc[pre] = (uint16_t)(off ? dict[x - 1] : PC_VAR);
        }
    }
};

// Emission order: the last phrase first (its next-suffix rank is -1,
// K:787-807), then the phrase before each parse suffix in suffix-array order.
struct Emit {
    const uint32_t *psa, *pisa, *pid, *moff, *D;
    uint32_t z;
    __device__ __forceinline__ uint32_t occ_at(size_t t) const
    {
        if (t == 0) return z - 1u;
        const uint32_t pos0 = pisa[0];
        const uint32_t r = (uint32_t)t - 1u < pos0 ? (uint32_t)t - 1u : (uint32_t)t;
        return psa[r] - 1u;
    }
};

// Per emission slot t: phrase id, number of mixed elements and the byte
// preceding the occurrence (the random gathers happen once, here).
__global__ void k_emit_prep(Emit e, const uint32_t *pidpc, const uint8_t *T, uint32_t n, int W, uint32_t *emq,
                            uint8_t *emp, uint32_t *ecnt)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= e.z) return;
    const uint32_t k = e.occ_at(t);
    uint32_t q, prev;
    if (pidpc) {                      // one gather: id and preceding byte packed
        const uint32_t v = pidpc[k];
        q = v >> 8;
        prev = v & 0xFFu;
    } else {
        q = e.pid[k];
        const uint32_t start = k ? e.D[k - 1] - (uint32_t)W + 1u : 0u;
        prev = preceding_byte(T, n, start);
    }
    emq[t] = q;
    emp[t] = (uint8_t)prev;
    ecnt[t] = e.moff[q + 1] - e.moff[q];
}

// 256 emission slots per CTA; the CTA writes its contiguous output range
// with consecutive threads on consecutive elements.
constexpr int EM_T = 256;
constexpr int EM_PER = 8;          // consecutive elements per thread and chunk
template <typename E>
__global__ void __launch_bounds__(EM_T) k_emit(uint32_t z, const uint32_t *eoff, const uint32_t *emq,
                                               const uint8_t *emp, const uint32_t *moff, const uint32_t *mb,
                                               const uint16_t *mc, E *elem, uint32_t cap, uint32_t *flags)
{
    __shared__ uint32_t s_off[EM_T + 1];
    __shared__ uint32_t s_base[EM_T];
    __shared__ uint8_t s_prev[EM_T];
    __shared__ E s_out[EM_T * EM_PER + EM_T * EM_PER / 32];     // sc_pad layout (bank-conflict free)
    const uint32_t t0 = blockIdx.x * EM_T;
    const uint32_t tn = min((uint32_t)EM_T, z - t0);
    if (threadIdx.x < tn) {
        const uint32_t t = t0 + threadIdx.x;
        s_off[threadIdx.x] = eoff[t];
        s_base[threadIdx.x] = moff[emq[t]];
        s_prev[threadIdx.x] = emp[t];
    }
    if (threadIdx.x == 0) s_off[tn] = eoff[t0 + tn];
    __syncthreads();
    const uint32_t o0 = s_off[0], cnt = s_off[tn] - o0;
    if ((uint64_t)o0 + cnt > cap) {
        if (threadIdx.x == 0) atomicOr(flags, ERR_INTERNAL);
        return;
    }
    // chunks of EM_T * EM_PER elements: each thread finds the slot of its
    // first element once and walks forward; the chunk is staged in shared
    // memory and written with consecutive threads on consecutive elements
    for (uint32_t cb = 0; cb < cnt; cb += EM_T * EM_PER) {
        const uint32_t e0 = cb + threadIdx.x * EM_PER;
        if (e0 < cnt) {
            const uint32_t o = o0 + e0;
            uint32_t lo = 0, hi = tn - 1u;            // last slot with s_off <= o
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1u) >> 1;
                if (s_off[mid] <= o) lo = mid; else hi = mid - 1u;
            }
#pragma unroll
            for (int q = 0; q < EM_PER; q++) {
                const uint32_t e = e0 + q;
                if (e >= cnt) break;
                while (s_off[lo + 1] <= o0 + e) lo++;
                const uint32_t j = s_base[lo] + (o0 + e - s_off[lo]);
                uint32_t c = mc[j];
                if (c == PC_VAR) c = s_prev[lo];
                s_out[sc_pad(threadIdx.x * EM_PER + q)] = ((E)mb[j] << 8) | (E)c;
            }
        }
        __syncthreads();
        const uint32_t m = min((uint32_t)(EM_T * EM_PER), cnt - cb);
        for (uint32_t i = threadIdx.x; i < m; i += EM_T) elem[o0 + cb + i] = s_out[sc_pad(i)];
        __syncthreads();
    }
}

// 4 sorted elements per thread; consecutive elements of one block land on
// consecutive output bytes.
template <typename E>
__global__ void k_mixed_scatter(const E *elem, uint32_t M, const uint32_t *delta, uint32_t B, uint8_t *out,
                                uint32_t n, uint32_t *flags)
{
    const uint32_t i0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4u;
    if (i0 >= M) return;
    E v[4];
    if (i0 + 4u <= M) {                 // one (or two) 16-byte loads
        if constexpr (sizeof(E) == 4) {
            const uint4 w = *(const uint4 *)(elem + i0);
            memcpy(v, &w, 16);
        } else {
            const ulonglong2 w0 = *(const ulonglong2 *)(elem + i0);
            const ulonglong2 w1 = *(const ulonglong2 *)(elem + i0 + 2);
            memcpy(v, &w0, 16);
            memcpy((char *)v + 16, &w1, 16);
        }
    } else {
#pragma unroll
        for (uint32_t j = 0; j < 4; j++) v[j] = i0 + j < M ? elem[i0 + j] : (E)0;
    }
#pragma unroll
    for (uint32_t j = 0; j < 4; j++) {
        const uint32_t i = i0 + j;
        if (i >= M) break;
        const E e = v[j];
        const uint32_t b = (uint32_t)(e >> 8);
        const uint32_t p = b < B ? i + delta[b] : 0xFFFFFFFFu;
        if (p < n) out[p] = (uint8_t)(e & 0xFFu);
        else atomicOr(flags, ERR_INTERNAL);
    }
}

// Run fill, one thread per group: the block [goff[g], goff[g+1]) of a run
// group is one byte repeated; the thread writes the bytes up to the first
// 16-byte boundary one by one, the middle with 16-byte stores and the tail
// one by one (neighbouring threads' edge bytes meet in L2).  Mixed groups are
// skipped: the mixed scatter writes every byte of theirs.  Blocks longer than
// RF_LONG bytes are listed and filled by one CTA each, so no thread carries a
// long block.
constexpr uint32_t RF_LONG = 512;

__device__ __forceinline__ void fill_run(uint8_t *out, uint32_t b0, uint32_t b1, uint8_t c)
{
    uint32_t p = b0;
    while (p < b1 && (((uintptr_t)(out + p)) & 15u)) out[p++] = c;
    const uint32_t w = (uint32_t)c * 0x01010101u;
    const uint4 v = make_uint4(w, w, w, w);
    for (; p + 16u <= b1; p += 16u) *(uint4 *)(out + p) = v;
    for (; p < b1; p++) out[p] = c;
}

__global__ void k_run_fill_groups(uint8_t *out, uint32_t n, const uint32_t *goff, uint32_t G, const uint16_t *gchar,
                                  const uint8_t *gmix, uint32_t *longs, uint32_t long_cap, uint32_t *flags)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G || gmix[g]) return;
    const uint32_t b0 = goff[g], b1 = goff[g + 1];
    if (b1 < b0 || b1 > n) { atomicOr(flags, ERR_INTERNAL); return; }
    if (b1 - b0 > RF_LONG) {
        const uint32_t i = atomicAdd(flags + 5, 1u);
        if (i < long_cap) longs[i] = g;
        else atomicOr(flags, ERR_INTERNAL);
        return;
    }
    fill_run(out, b0, b1, (uint8_t)gchar[g]);
}

// One CTA per listed long run (the count is read on the device: no host sync).
__global__ void k_run_fill_long(uint8_t *out, const uint32_t *goff, const uint16_t *gchar, const uint32_t *longs,
                                const uint32_t *nlong, uint32_t long_cap)
{
    const uint32_t cnt = min(*nlong, long_cap);
    for (uint32_t i = blockIdx.x; i < cnt; i += gridDim.x) {
        const uint32_t g = longs[i];
        const uint32_t b0 = goff[g], b1 = goff[g + 1];
        const uint8_t c = (uint8_t)gchar[g];
        // head bytes to the first 16-byte boundary, then striped 16-byte stores
        uint32_t a0 = b0;
        while (a0 < b1 && (((uintptr_t)(out + a0)) & 15u)) a0++;
        if (threadIdx.x < a0 - b0) out[b0 + threadIdx.x] = c;
        const uint32_t nv = (b1 - a0) / 16u;
        const uint32_t w = (uint32_t)c * 0x01010101u;
        const uint4 v = make_uint4(w, w, w, w);
        for (uint32_t j = threadIdx.x; j < nv; j += blockDim.x) *(uint4 *)(out + a0 + 16u * j) = v;
        const uint32_t t0 = a0 + 16u * nv;
        if (threadIdx.x < b1 - t0) out[t0 + threadIdx.x] = c;
    }
}

// Output row of the suffix starting at text position 0 (the "primary index"):
// its block is the group g0 of phrase 0 taken whole; inside a block the rows
// follow the rank of the next parse suffix (last phrase: -1, K:787-807).
struct PrimaryArgs {
    const uint32_t *pid, *pisa, *doff, *dlen, *grp_of, *goff;
    uint32_t z;
    uint32_t *counter;
};
__global__ void k_primary_index(PrimaryArgs a)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t q0 = a.pid[0], len0 = a.dlen[q0];
    const uint32_t g0 = a.grp_of[a.doff[q0]];
    bool before = false;
    if (k < a.z && k != 0) {
        const uint32_t q = a.pid[k], lq = a.dlen[q];
        if (lq >= len0 && a.grp_of[a.doff[q] + lq - len0] == g0) {
            const int64_t nr0 = a.z > 1 ? (int64_t)a.pisa[1] : -1;
            const int64_t nrk = k + 1 < a.z ? (int64_t)a.pisa[k + 1] : -1;
            before = nrk < nr0;
        }
    }
    const unsigned m = __ballot_sync(0xFFFFFFFFu, before);
    if ((threadIdx.x & 31u) == 0 && m) atomicAdd(a.counter, (uint32_t)__popc(m));
    if (k == 0) atomicAdd(a.counter, a.goff[g0]);
}

template <typename E>
static void mixed_blocks(Storage *st, const uint8_t *dT, uint32_t n, int W, Phrases &ph, ParseOrder &pord,
                         const uint32_t *moff, const uint32_t *mb, const uint16_t *mc, const uint32_t *delta,
                         uint32_t B, uint32_t M, uint8_t *dOut)
{
    E *elem = slot<E>(st, S_ELEM0, M);
    E *elem_alt = slot<E>(st, S_ELEM1, M);
    const uint32_t z = ph.z;
    Emit e{pord.sa, pord.isa, ph.pid, moff, ph.D, z};
    uint32_t *emq = slot<uint32_t>(st, S_TMP0, z);
    uint32_t *ecnt = slot<uint32_t>(st, S_TMP1, (size_t)z + 1);
    uint8_t *emp = (uint8_t *)slot<uint32_t>(st, S_TMP2, z / 4 + 1);
    k_emit_prep<<<grid_for(z, 256), 256, 0, st->stream>>>(e, ph.pidpc, dT, n, W, emq, emp, ecnt);
    after_launch(st);
    // in-place exclusive scan of the counts; ecnt[z] = total
    device_scan<uint32_t, OpAdd>(st, z, LoadArr<uint32_t>{ecnt}, StoreArr<uint32_t>{ecnt}, false, ecnt + z);
    k_emit<E><<<grid_for(z, EM_T), EM_T, 0, st->stream>>>(z, ecnt, emq, emp, moff, mb, mc, elem, M, st->d_flags);
    after_launch(st);
    uint32_t *nv = nullptr, *nv2 = nullptr;
    // sort by block id; 8-bit digits unless the tuning asks for 10 (fewer
    // passes, larger tile histograms)
    if (st->tuning.mixed_radix_bits == 10) radix_sort<E, false, 10>(st, elem, elem_alt, nv, nv2, M, 8, 8 + bits_for(B - 1));
    else radix_sort<E, false, 8>(st, elem, elem_alt, nv, nv2, M, 8, 8 + bits_for(B - 1));
    probe_begin(st, GBWT_PROBE_MIXED_SCATTER);
    k_mixed_scatter<E><<<grid_for((M + 3) / 4, 256), 256, 0, st->stream>>>(elem, M, delta, B, dOut, n, st->d_flags);
    probe_end(st, GBWT_PROBE_MIXED_SCATTER, (uint64_t)M * (sizeof(E) + 1));
    after_launch(st);
}

uint32_t run_group_index(Storage *st, Phrases &ph, DictOrder &dord, int W, uint32_t *&grp_of)
{
    const uint32_t N = (uint32_t)ph.dict_bytes;
    PosInfo pi{ph.dphr, ph.doff, ph.dlen};
    uint32_t *gid = nullptr;
    const uint32_t G = group_numbers(st, ph, dord, W, gid);
    grp_of = slot<uint32_t>(st, S_GRP, N);
    k_group_of<<<grid_for(N, 256), 256, 0, st->stream>>>(N, pi, (uint32_t)W, dord.isa, gid, grp_of, nullptr,
                                                         nullptr, nullptr, nullptr, nullptr, nullptr);
    after_launch(st);
    return G;
}

void run_assembly(Storage *st, const uint8_t *dT, uint32_t n, int W, Phrases &ph, DictOrder &dord,
                  ParseOrder &pord, uint8_t *dOut)
{
    const uint32_t N = (uint32_t)ph.dict_bytes;
    PosInfo pi{ph.dphr, ph.doff, ph.dlen};
    // groups: at most one per dictionary position
    uint32_t *gcount = slot<uint32_t>(st, S_GCOUNT, N);
    uint16_t *gchar = slot<uint16_t>(st, S_GCHAR, N);
    uint32_t *grp_of = slot<uint32_t>(st, S_GRP, N);
    uint32_t *gid = nullptr;
    const uint32_t G = group_numbers(st, ph, dord, W, gid);
    if (G == 0) throw Error{GBWT_INTERNAL_ERROR};
    check_cuda(cudaMemsetAsync(gcount, 0, (size_t)G * 4, st->stream));
    k_group_of<<<grid_for(N, 256), 256, 0, st->stream>>>(N, pi, (uint32_t)W, dord.isa, gid, grp_of, ph.dict, ph.occ,
                                                         ph.pcmin, ph.pcmax, gcount, gchar);
    after_launch(st);
    uint8_t *gmix = slot<uint8_t>(st, S_GMIX, G);
    check_cuda(cudaMemsetAsync(gmix, 0, G, st->stream));
    k_mark_mixed<<<grid_for(N, 256), 256, 0, st->stream>>>(N, pi, (uint32_t)W, ph.dict, ph.pcmin, ph.pcmax, grp_of,
                                                           gchar, gmix);
    after_launch(st);
    uint32_t *goff = slot<uint32_t>(st, S_GOFF, (size_t)G + 1);
    device_scan<uint32_t, OpAdd>(st, G, LoadGCount{gcount}, StoreArr<uint32_t>{goff}, false, goff + G);
    uint32_t *mixidx = slot<uint32_t>(st, S_MIXIDX, G);
    uint32_t *delta = slot<uint32_t>(st, S_DELTA, G);
    check_cuda(cudaMemsetAsync(st->d_scalars + 1, 0, 8, st->stream));
    device_scan<uint64_t, OpAdd>(st, G, LoadMixPair{gcount, gmix}, StoreMix{gmix, goff, mixidx, delta}, false,
                                 (uint64_t *)(st->d_scalars + 1));
    check_cuda(cudaMemcpyAsync(st->d_scalars + 2, goff + G, 4, cudaMemcpyDeviceToDevice, st->stream));
    fetch_scalars(st, 3);
    const uint32_t B = (uint32_t)(st->h_scalars[1] >> 32);
    const uint32_t M = (uint32_t)st->h_scalars[1];
    const uint32_t total = (uint32_t)st->h_scalars[2];
    if (total != n) throw Error{GBWT_INTERNAL_ERROR};
    st->stats.s = G;
    st->stats.mixed_blocks = B;
    st->stats.mixed_elems = M;
    stage_mark(st, 4);

    k_primary_index<<<grid_for(ph.z, 256), 256, 0, st->stream>>>(
        PrimaryArgs{ph.pid, pord.isa, ph.doff, ph.dlen, grp_of, goff, ph.z, st->d_flags + 2});
    after_launch(st);
    const uint32_t long_cap = n / RF_LONG + 1u;
    uint32_t *longs = slot<uint32_t>(st, S_TILEG, long_cap);
    check_cuda(cudaMemsetAsync(st->d_flags + 5, 0, 4, st->stream));
    probe_begin(st, GBWT_PROBE_RUN_FILL);
    k_run_fill_groups<<<grid_for(G, 256), 256, 0, st->stream>>>(dOut, n, goff, G, gchar, gmix, longs, long_cap,
                                                                st->d_flags);
    probe_end(st, GBWT_PROBE_RUN_FILL, (uint64_t)(n - M) + 7ull * G);
    after_launch(st);
    k_run_fill_long<<<st->num_sms * 4, 256, 0, st->stream>>>(dOut, goff, gchar, longs, st->d_flags + 5, long_cap);
    after_launch(st);
    stage_mark(st, 5);
    if (B == 0) return;

    // per-phrase mixed-suffix lists
    uint32_t *moff = slot<uint32_t>(st, S_MOFF, (size_t)ph.d + 1);
    uint32_t *mb = slot<uint32_t>(st, S_MB, N);
    uint16_t *mc = slot<uint16_t>(st, S_MC, N);
    device_scan<uint32_t, OpAdd>(st, N, LoadMixEntry{pi, (uint32_t)W, grp_of, gmix},
                                 StoreMixEntry{pi, ph.dict, grp_of, mixidx, moff, mb, mc}, false, moff + ph.d);
    if (B < (1u << 24)) mixed_blocks<uint32_t>(st, dT, n, W, ph, pord, moff, mb, mc, delta, B, M, dOut);
    else mixed_blocks<uint64_t>(st, dT, n, W, ph, pord, moff, mb, mc, delta, B, M, dOut);
}

}  // namespace gbwt
