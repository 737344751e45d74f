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
constexpr uint32_t PC_CHUNK = 16384;      // input bytes per CTA of the padded copy

// X[xstart[t] + i] = Tin[ioff[t] + i]; W sentinel bytes after each text.
// Consecutive threads copy consecutive bytes (the shift per text is arbitrary).
__global__ void __launch_bounds__(PC_THREADS) k_pad_copy(const uint8_t *Tin, uint64_t total, const uint32_t *ioff,
                                                         const uint32_t *xstart, uint32_t k, int W, uint32_t hi,
                                                         uint8_t *X, uint32_t *flags)
{
    __shared__ uint32_t s_t;
    const uint64_t c0 = (uint64_t)blockIdx.x * PC_CHUNK;
    const uint64_t c1 = c0 + PC_CHUNK < total ? c0 + PC_CHUNK : total;
    if (threadIdx.x == 0) {                 // last text with ioff <= c0
        uint32_t lo = 0, h = k - 1u;
        while (lo < h) {
            const uint32_t mid = (lo + h + 1u) >> 1;
            if (ioff[mid] <= c0) lo = mid; else h = mid - 1u;
        }
        s_t = lo;
    }
    __syncthreads();
    bool bad = false, small_bad = false;
    for (uint32_t t = s_t; t < k; t++) {
        const uint64_t a = ioff[t];
        if (a >= c1) break;
        const uint32_t xs = xstart[t];
        const uint32_t len = xstart[t + 1] - xs - (uint32_t)W;
        const uint64_t e = a + len;
        const uint64_t lo = a > c0 ? a : c0, up = e < c1 ? e : c1;
        for (uint64_t i = lo + threadIdx.x; i < up; i += PC_THREADS) {
            const uint32_t c = __ldg(Tin + i);
            bad |= (c < 2u) || (c == 255u);
            small_bad |= c > hi;
            X[xs + (uint32_t)(i - a)] = (uint8_t)c;
        }
        if (e > c0 && e <= c1 && threadIdx.x < (unsigned)W) X[xs + len + threadIdx.x] = 1;
    }
    const bool any_bad = __any_sync(0xFFFFFFFFu, bad), any_small = __any_sync(0xFFFFFFFFu, small_bad);
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

// Emission slots: k empty parse suffixes (slot t stands for the last phrase
// of text t), then the parse suffix array; slot of suffix x stands for the
// phrase before it, none when x starts its text.
struct BatchEmit {
    const uint32_t *psa, *pid, *pidpc, *D, *ptid, *zend, *dlen, *doff;
    const uint8_t *X, *lastb;
    uint32_t k, z;
    int W;
};

__global__ void k_bemit_prep(BatchEmit e, uint32_t *emq, uint32_t *emt, uint8_t *emp, uint32_t *ecnt)
{
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= e.k + e.z) return;
    uint32_t occ;
    if (s < e.k) {
        occ = e.zend[s] - 1u;
    } else {
        const uint32_t x = e.psa[s - e.k];
        if (x == 0 || e.ptid[x - 1] != e.ptid[x]) {
            emq[s] = 0; emt[s] = 0; emp[s] = 0; ecnt[s] = 0;
            return;
        }
        occ = x - 1u;
    }
    uint32_t q, prev;
    if (e.pidpc) {
        const uint32_t v = e.pidpc[occ];
        q = v >> 8;
        prev = v & 0xFFu;
    } else {
        q = e.pid[occ];
        const bool first = occ == 0 || e.X[e.D[occ - 1]] == 1;
        prev = first ? e.lastb[e.ptid[occ]] : e.X[e.D[occ - 1] - (uint32_t)e.W];
    }
    emq[s] = e.doff[q];
    emt[s] = e.ptid[occ];
    emp[s] = (uint8_t)prev;
    ecnt[s] = e.dlen[q] - (uint32_t)e.W;
}

// 256 slots per CTA; consecutive threads write consecutive elements.
constexpr int BE_T = 256;
__global__ void __launch_bounds__(BE_T) k_bemit(uint32_t S, const uint32_t *eoff, const uint32_t *emq,
                                                const uint32_t *emt, const uint8_t *emp, const uint32_t *grp_of,
                                                const uint8_t *dict, int gb, uint64_t *elem, uint32_t cap,
                                                uint32_t *flags)
{
    __shared__ uint32_t s_off[BE_T + 1];
    __shared__ uint32_t s_base[BE_T];
    __shared__ uint64_t s_hi[BE_T];
    __shared__ uint8_t s_prev[BE_T];
    const uint32_t t0 = blockIdx.x * BE_T;
    const uint32_t tn = min((uint32_t)BE_T, S - t0);
    if (threadIdx.x < tn) {
        const uint32_t t = t0 + threadIdx.x;
        s_off[threadIdx.x] = eoff[t];
        s_base[threadIdx.x] = emq[t];
        s_hi[threadIdx.x] = (uint64_t)emt[t] << gb;
        s_prev[threadIdx.x] = emp[t];
    }
    if (threadIdx.x == 0) s_off[tn] = eoff[t0 + tn];
    __syncthreads();
    const uint32_t o0 = s_off[0], cnt = s_off[tn] - o0;
    if ((uint64_t)o0 + cnt > cap) {
        if (threadIdx.x == 0) atomicOr(flags, ERR_INTERNAL);
        return;
    }
    for (uint32_t i = threadIdx.x; i < cnt; i += BE_T) {
        const uint32_t o = o0 + i;
        uint32_t lo = 0, hi = tn - 1u;            // last slot with s_off <= o
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1u) >> 1;
            if (s_off[mid] <= o) lo = mid; else hi = mid - 1u;
        }
        const uint32_t j = o - s_off[lo];
        const uint32_t pos = s_base[lo] + j;
        const uint32_t c = j ? dict[pos - 1] : s_prev[lo];
        elem[o] = ((s_hi[lo] | grp_of[pos]) << 8) | c;
    }
}

// Output bytes = the low byte of the sorted elements, 16 per thread.
__global__ void k_extract(const uint64_t *elem, uint32_t n, uint8_t *out)
{
    const uint32_t i0 = (blockIdx.x * blockDim.x + threadIdx.x) * 16u;
    if (i0 >= n) return;
    if (i0 + 16u <= n && (((uintptr_t)(out + i0)) & 15u) == 0) {
        uint8_t b[16];
#pragma unroll
        for (int j = 0; j < 16; j++) b[j] = (uint8_t)elem[i0 + j];
        uint4 v;
        memcpy(&v, b, 16);
        *(uint4 *)(out + i0) = v;
    } else {
        for (uint32_t j = 0; j < 16 && i0 + j < n; j++) out[i0 + j] = (uint8_t)elem[i0 + j];
    }
}

// Texts with offsets[t] < offsets[t+1]; their layout in X.  Returns the
// number of non-empty texts; h_meta receives xstart[k'+1] then ioff[k'].
static uint32_t batch_layout(Storage *st, const int64_t *offsets, int32_t k, int W, uint64_t &total, uint64_t &N)
{
    total = (uint64_t)offsets[k];
    uint32_t kk = 0;
    for (int32_t t = 0; t < k; t++) kk += offsets[t + 1] > offsets[t] ? 1u : 0u;
    const size_t need = (size_t)2 * kk + 1;
    if (st->h_meta_cap < need) {
        if (st->h_meta) check_cuda(cudaFreeHost(st->h_meta));
        st->h_meta = nullptr;
        st->h_meta_cap = 0;
        size_t cap = need + need / 4 + 1024;
        check_cuda(cudaHostAlloc(&st->h_meta, cap * sizeof(uint32_t), cudaHostAllocDefault));
        st->h_meta_cap = cap;
    }
    uint32_t *xs = st->h_meta, *io = st->h_meta + kk + 1;
    uint32_t i = 0;
    uint64_t x = 0;
    for (int32_t t = 0; t < k; t++) {
        const uint64_t len = (uint64_t)(offsets[t + 1] - offsets[t]);
        if (!len) continue;
        xs[i] = (uint32_t)x;
        io[i] = (uint32_t)offsets[t];
        x += len + (uint64_t)W;
        i++;
    }
    xs[kk] = (uint32_t)x;
    N = x;
    return kk;
}

int64_t run_batch(Storage *st, const uint8_t *T, const int64_t *offsets, int32_t k, uint8_t *L, int W, int P,
                  uint32_t flags, int64_t max_n)
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
    uint64_t total = 0, N = 0;
    // 32-bit positions inside, with room for the sentinel runs
    if ((uint64_t)total_i + (uint64_t)W * (uint64_t)k > (uint64_t)max_n) return GBWT_UNSUPPORTED_INPUT;
    const uint32_t kk = batch_layout(st, offsets, k, W, total, N);

    uint32_t *meta = slot<uint32_t>(st, S_BMETA, (size_t)2 * kk + 1);
    check_cuda(cudaMemcpyAsync(meta, st->h_meta, ((size_t)2 * kk + 1) * 4, cudaMemcpyHostToDevice, st->stream));
    const uint32_t *xstart = meta, *ioff = meta + kk + 1;
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
    k_pad_copy<<<grid_for(total, PC_CHUNK), PC_THREADS, 0, st->stream>>>(dT, total, ioff, xstart, kk, W,
                                                                         small ? 15u : 254u, X, st->d_flags);
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
    stage_mark(st, 2);

    ParseOrder pord;
    run_parse_sa_batch(st, ph, dord, bt, pord);
    st->stats.parse_rounds = pord.rounds;
    stage_mark(st, 3);

    uint32_t *grp_of = nullptr;
    const uint32_t G = run_group_index(st, ph, dord, W, grp_of);
    if (G == 0) throw Error{GBWT_INTERNAL_ERROR};
    st->stats.s = G;
    const int tb = bits_for(kk - 1u), gb = bits_for(G - 1u);
    if (8 + tb + gb > 64) throw Error{GBWT_UNSUPPORTED_INPUT};
    stage_mark(st, 4);

    const uint32_t S = kk + z;
    uint32_t *emq = slot<uint32_t>(st, S_TMP0, S);
    uint32_t *emt = slot<uint32_t>(st, S_TMP1, S);
    uint8_t *emp = slot<uint8_t>(st, S_TMP2, S);
    uint32_t *ecnt = slot<uint32_t>(st, S_GCOUNT, (size_t)S + 1);
    BatchEmit e{pord.sa, ph.pid, ph.pidpc, ph.D, ptid, zend, ph.dlen, ph.doff, X, lastb, kk, z, W};
    k_bemit_prep<<<grid_for(S, 256), 256, 0, st->stream>>>(e, emq, emt, emp, ecnt);
    after_launch(st);
    device_scan<uint32_t, OpAdd>(st, S, LoadArr<uint32_t>{ecnt}, StoreArr<uint32_t>{ecnt}, false, ecnt + S);
    check_cuda(cudaMemcpyAsync(st->d_scalars, ecnt + S, 4, cudaMemcpyDeviceToDevice, st->stream));
    fetch_scalars(st, 1);
    if ((uint32_t)st->h_scalars[0] != (uint32_t)total) throw Error{GBWT_INTERNAL_ERROR};
    const uint32_t M = (uint32_t)total;
    uint64_t *elem = slot<uint64_t>(st, S_ELEM0, M);
    uint64_t *elem_alt = slot<uint64_t>(st, S_ELEM1, M);
    k_bemit<<<grid_for(S, BE_T), BE_T, 0, st->stream>>>(S, ecnt, emq, emt, emp, grp_of, ph.dict, gb, elem, M,
                                                        st->d_flags);
    after_launch(st);
    uint32_t *nv = nullptr, *nv2 = nullptr;
    radix_sort<uint64_t, false, 8>(st, elem, elem_alt, nv, nv2, M, 8, 8 + tb + gb);
    stage_mark(st, 5);
    k_extract<<<grid_for(M, 256 * 16), 256, 0, st->stream>>>(elem, M, dOut);
    after_launch(st);
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
