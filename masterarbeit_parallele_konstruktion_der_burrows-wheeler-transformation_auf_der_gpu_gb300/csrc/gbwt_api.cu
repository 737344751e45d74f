// gbwt_api.cu -- C ABI of the PFP BWT library and the host-side pipeline.
//
// The pipeline mirrors the reference's main() (Prefix_Free_Parsing_W=5_P=16
// _kommentiert.cu, "K", K:4793-4815): input -> phrase ends (Compute_D,
// K:2415-2506) -> dictionary / parse / S / blocks (Compute_S, K:4330-4771)
// -> output.  All device work is stream-ordered on the storage's stream;
// host synchronisation happens only where a size decides the next launch.
#include "prims.cuh"
#include <new>
#include <stdio.h>
#include <stdlib.h>
#include <vector>

namespace gbwt {

void stage_mark(Storage *st, int idx)
{
    if (st->stage_times) check_cuda(cudaEventRecord(st->ev[idx + 1], st->stream));
}

__global__ void k_gather_ranks(const uint32_t *pid, const uint32_t *lexrank, uint32_t z, uint32_t *out)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < z) out[k] = lexrank[pid[k]];
}

// Adds the recorded probe event pairs (the stream is idle) to the totals.
static void harvest_probe(Storage *st)
{
    for (int i = 0; i < st->probe_used; i++) {
        float ms = 0.f;
        check_cuda(cudaEventElapsedTime(&ms, st->probe_ev[2 * i], st->probe_ev[2 * i + 1]));
        st->probe_ms += ms;
    }
    st->probe_used = 0;
    st->stats.probe_launches = st->probe_launches;
    st->stats.probe_bytes = st->probe_bytes;
    st->stats.probe_ms = st->probe_ms;
}

enum Upto { UPTO_SCAN = 0, UPTO_PARSE = 1, UPTO_BWT = 2 };

struct StageOut {
    int64_t *D = nullptr;
    int32_t *ranks = nullptr;
    int32_t *parse_sa = nullptr;
    int64_t capacity = 0;
};

static const int64_t MAX_N = 0x7FFFFFFFll - 128;   // 32-bit positions inside

static int64_t pipeline(Storage *st, const uint8_t *T, uint8_t *L, int64_t n, int32_t W, int32_t P, uint32_t flags,
                        Upto upto, StageOut *so)
{
    if (n < 0 || n > MAX_N || W < 1 || W > 64 || P < 1 || P > 65535) return GBWT_BAD_PARAMETER;
    if (n > 0 && !T) return GBWT_BAD_PARAMETER;
    if (upto == UPTO_BWT && n > 0 && !L) return GBWT_BAD_PARAMETER;
    const bool small = (flags & GBWT_FLAG_SMALL_ALPHABET) != 0;
    const bool devptr = (flags & GBWT_FLAG_DEVICE_POINTERS) != 0;
    memset(&st->stats, 0, sizeof(st->stats));
    st->launches = 0;
    st->stats.n = n;
    st->stage_times = (flags & GBWT_FLAG_STAGE_TIMES) != 0;
    if (n == 0) return 0;
    const uint32_t un = (uint32_t)n;

    const uint8_t *dT;
    uint8_t *dOut = nullptr;
    if (devptr) {
        dT = T;
        dOut = L;
    } else {
        uint8_t *buf = slot<uint8_t>(st, S_TEXT, (size_t)n + 16);
        check_cuda(cudaMemcpyAsync(buf, T, (size_t)n, cudaMemcpyHostToDevice, st->stream));
        dT = buf;
        if (upto == UPTO_BWT) dOut = slot<uint8_t>(st, S_OUT, (size_t)n + 16);
    }
    if (st->stage_times) check_cuda(cudaEventRecord(st->ev[0], st->stream));
    check_cuda(cudaMemsetAsync(st->d_flags, 0, 64 * sizeof(uint32_t), st->stream));

    uint32_t *D = nullptr;
    const uint32_t z = run_trigger_scan(st, dT, un, W, P, small, D);
    st->stats.z = z;
    stage_mark(st, 0);
    if (upto == UPTO_SCAN) {
        if ((int64_t)z > so->capacity) return GBWT_BAD_PARAMETER;
        std::vector<uint32_t> h(z);
        check_cuda(cudaMemcpyAsync(h.data(), D, (size_t)z * 4, cudaMemcpyDeviceToHost, st->stream));
        check_cuda(cudaStreamSynchronize(st->stream));
        for (uint32_t i = 0; i < z; i++) so->D[i] = h[i];
        st->stats.kernel_launches = st->launches;
        return z;
    }

    Phrases ph;
    ph.z = z;
    ph.D = D;
    run_phrases(st, dT, un, W, ph);
    st->stats.d = ph.d;
    st->stats.dict_bytes = (int64_t)ph.dict_bytes;
    stage_mark(st, 1);

    DictOrder dord;
    run_dict_sort(st, ph, W, small, dord);
    st->stats.dict_rounds = dord.rounds;
    stage_mark(st, 2);

    ParseOrder pord;
    run_parse_sa(st, ph, dord, pord);
    st->stats.parse_rounds = pord.rounds;
    stage_mark(st, 3);

    if (upto == UPTO_PARSE) {
        if ((int64_t)z > so->capacity) return GBWT_BAD_PARAMETER;
        uint32_t *tmp = slot<uint32_t>(st, S_TMP1, z);
        k_gather_ranks<<<grid_for(z, 256), 256, 0, st->stream>>>(ph.pid, dord.lexrank, z, tmp);
        after_launch(st);
        std::vector<uint32_t> h(z), h2;
        check_cuda(cudaMemcpyAsync(h.data(), tmp, (size_t)z * 4, cudaMemcpyDeviceToHost, st->stream));
        if (so->parse_sa) {
            h2.resize(z);
            check_cuda(cudaMemcpyAsync(h2.data(), pord.sa, (size_t)z * 4, cudaMemcpyDeviceToHost, st->stream));
        }
        check_cuda(cudaStreamSynchronize(st->stream));
        for (uint32_t i = 0; i < z; i++) so->ranks[i] = (int32_t)h[i];
        if (so->parse_sa)
            for (uint32_t i = 0; i < z; i++) so->parse_sa[i] = (int32_t)h2[i];
        st->stats.kernel_launches = st->launches;
        return z;
    }

    run_assembly(st, dT, un, W, ph, dord, pord, dOut);
    stage_mark(st, 6);
    if (!devptr) check_cuda(cudaMemcpyAsync(L, dOut, (size_t)n, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaMemcpyAsync(st->h_scalars + 8, st->d_flags, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                               st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    uint32_t hflags[4];
    memcpy(hflags, st->h_scalars + 8, sizeof(hflags));
    if (hflags[0] & ERR_TIMEOUT) return GBWT_TIMEOUT;
    if (hflags[0] & ERR_INTERNAL) return GBWT_INTERNAL_ERROR;
    st->stats.primary_index = hflags[2];
    harvest_probe(st);
    if (st->stage_times) {
        // stages 4/5 may be skipped (no mixed blocks): fall back to the previous mark
        for (int i = 0; i < 7; i++) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, st->ev[i], st->ev[i + 1]) != cudaSuccess) ms = 0.f;
            st->stats.stage_ms[i] = ms;
        }
        float tot = 0.f;
        if (cudaEventElapsedTime(&tot, st->ev[0], st->ev[7]) == cudaSuccess) st->stats.stage_ms[7] = tot;
    }
    st->stats.kernel_launches = st->launches;
    return n;
}

template <typename F>
static int64_t guarded(F f)
{
    try {
        return f();
    } catch (const Error &e) {
        return e.code;
    } catch (const std::bad_alloc &) {
        return GBWT_NOT_ENOUGH_MEMORY;
    } catch (...) {
        return GBWT_INTERNAL_ERROR;
    }
}

}  // namespace gbwt

using namespace gbwt;

extern "C" int64_t gbwt_allocate_device_storage(void **storage, int64_t max_length)
{
    if (!storage || max_length < 0 || max_length > MAX_N) return GBWT_BAD_PARAMETER;
    *storage = nullptr;
    Storage *st = new (std::nothrow) Storage();
    if (!st) return GBWT_NOT_ENOUGH_MEMORY;
    int64_t rc = guarded([&]() -> int64_t {
        check_cuda(cudaGetDevice(&st->device));
        int major = 0, minor = 0;
        check_cuda(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, st->device));
        check_cuda(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, st->device));
        if (major * 10 + minor != 103) return GBWT_GPU_NOT_SUPPORTED;   // built for sm_103a only
        check_cuda(cudaDeviceGetAttribute(&st->num_sms, cudaDevAttrMultiProcessorCount, st->device));
        check_cuda(cudaStreamCreateWithFlags(&st->own_stream, cudaStreamNonBlocking));
        st->stream = st->own_stream;
        check_cuda(cudaMalloc(&st->d_flags, 64 * sizeof(uint32_t)));
        check_cuda(cudaMalloc(&st->d_scalars, 64 * sizeof(uint64_t)));
        check_cuda(cudaHostAlloc(&st->h_scalars, 256 * sizeof(uint64_t), cudaHostAllocDefault));
        for (int i = 0; i < 10; i++) check_cuda(cudaEventCreate(&st->ev[i]));
        st->max_length = max_length;
        if (max_length > 0) {
            slot<uint8_t>(st, S_TEXT, (size_t)max_length + 16);
            slot<uint8_t>(st, S_OUT, (size_t)max_length + 16);
        }
        return GBWT_NO_ERROR;
    });
    if (rc != GBWT_NO_ERROR) {
        gbwt_free_device_storage(st);
        return rc;
    }
    *storage = st;
    return GBWT_NO_ERROR;
}

extern "C" int64_t gbwt_free_device_storage(void *storage)
{
    Storage *st = (Storage *)storage;
    if (!st) return GBWT_BAD_PARAMETER;
    cudaError_t err = cudaSuccess;
    if (st->stream) cudaStreamSynchronize(st->stream);
    for (int i = 0; i < S_NUM; i++)
        if (st->slots[i].p) {
            cudaError_t e = cudaFree(st->slots[i].p);
            if (e != cudaSuccess) err = e;
        }
    if (st->d_flags) cudaFree(st->d_flags);
    if (st->d_scalars) cudaFree(st->d_scalars);
    if (st->h_scalars) cudaFreeHost(st->h_scalars);
    if (st->h_meta) cudaFreeHost(st->h_meta);
    for (int i = 0; i < 10; i++)
        if (st->ev[i]) cudaEventDestroy(st->ev[i]);
    for (int i = 0; i < 2 * st->probe_cap; i++) cudaEventDestroy(st->probe_ev[i]);
    free(st->probe_ev);
    if (st->own_stream) cudaStreamDestroy(st->own_stream);
    delete st;
    return err == cudaSuccess ? GBWT_NO_ERROR : GBWT_GPU_ERROR;
}

extern "C" int64_t gbwt_set_stream(void *storage, void *cuda_stream)
{
    Storage *st = (Storage *)storage;
    if (!st) return GBWT_BAD_PARAMETER;
    st->stream = cuda_stream ? (cudaStream_t)cuda_stream : st->own_stream;
    return GBWT_NO_ERROR;
}

extern "C" int64_t gbwt_pfp_bwt(void *storage, const uint8_t *T, uint8_t *L, int64_t n, int32_t W, int32_t P,
                                uint32_t flags)
{
    Storage *st = (Storage *)storage;
    if (!st) return GBWT_BAD_PARAMETER;
    return guarded([&]() { return pipeline(st, T, L, n, W, P, flags, UPTO_BWT, nullptr); });
}

// Inverse BWT: the PFP output convention (primary = gbwt_stats.primary_index)
// or libcubwt's (its primary index, L without the '$' row).
static int64_t unbwt_common(Storage *st, const uint8_t *L, uint8_t *T, int64_t n, int64_t primary, bool pfp,
                            bool devptr)
{
    if (n < 0 || n > MAX_N) return GBWT_BAD_PARAMETER;
    if (n == 0) return 0;
    if (!L || !T) return GBWT_BAD_PARAMETER;
    if (pfp ? (primary < 0 || primary >= n) : (primary < 1 || primary > n)) return GBWT_BAD_PARAMETER;
    memset(&st->stats, 0, sizeof(st->stats));
    st->launches = 0;
    st->stats.n = n;
    const uint32_t un = (uint32_t)n;
    const uint8_t *dL;
    uint8_t *dT;
    if (devptr) {
        dL = L;
        dT = T;
    } else {
        uint8_t *buf = slot<uint8_t>(st, S_TEXT, (size_t)n + 16);
        check_cuda(cudaMemcpyAsync(buf, L, (size_t)n, cudaMemcpyHostToDevice, st->stream));
        dL = buf;
        dT = slot<uint8_t>(st, S_OUT, (size_t)n + 16);
    }
    check_cuda(cudaMemsetAsync(st->d_flags, 0, 64 * sizeof(uint32_t), st->stream));
    const uint8_t *dLc = dL;
    if (pfp) {
        uint8_t *lc = slot<uint8_t>(st, S_LCB, (size_t)n + 16);
        pfp_to_libcubwt(st, dL, un, (uint32_t)primary, lc);
        dLc = lc;
    }
    run_unbwt(st, dLc, un, pfp ? (uint32_t)primary + 1u : (uint32_t)primary, dT);
    if (!devptr) check_cuda(cudaMemcpyAsync(T, dT, (size_t)n, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaMemcpyAsync(st->h_scalars + 8, st->d_flags, 4, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    if ((uint32_t)st->h_scalars[8] & ERR_INTERNAL) return GBWT_INTERNAL_ERROR;
    st->stats.kernel_launches = st->launches;
    return n;
}

extern "C" int64_t gbwt_unbwt(void *storage, const uint8_t *L, uint8_t *T, int64_t n, int64_t primary, uint32_t flags)
{
    Storage *st = (Storage *)storage;
    if (!st) return GBWT_BAD_PARAMETER;
    return guarded([&]() {
        return unbwt_common(st, L, T, n, primary, true, (flags & GBWT_FLAG_DEVICE_POINTERS) != 0);
    });
}

extern "C" int64_t gbwt_libcubwt_unbwt(void *storage, const uint8_t *T, uint8_t *U, int64_t n, const int32_t *freq,
                                       int32_t i)
{
    (void)freq;       // recomputed on the device
    Storage *st = (Storage *)storage;
    if (!st) return GBWT_BAD_PARAMETER;
    return guarded([&]() -> int64_t {
        const int64_t rc = unbwt_common(st, T, U, n, i, false, false);
        return rc < 0 ? rc : GBWT_NO_ERROR;
    });
}

extern "C" int64_t gbwt_pfp_bwt_batch(void *storage, const uint8_t *T_concat, const int64_t *offsets, int32_t k,
                                      uint8_t *L_concat, int32_t W, int32_t P, uint32_t flags)
{
    Storage *st = (Storage *)storage;
    if (!st) return GBWT_BAD_PARAMETER;
    return guarded([&]() { return run_batch(st, T_concat, offsets, k, L_concat, W, P, flags, MAX_N); });
}

extern "C" int64_t gbwt_pfp_trigger_scan(void *storage, const uint8_t *T, int64_t n, int32_t W, int32_t P,
                                         uint32_t flags, int64_t *D, int64_t capacity)
{
    Storage *st = (Storage *)storage;
    if (!st || !D || capacity < 1) return GBWT_BAD_PARAMETER;
    StageOut so;
    so.D = D;
    so.capacity = capacity;
    if (n == 0) return 0;
    return guarded([&]() { return pipeline(st, T, nullptr, n, W, P, flags & ~GBWT_FLAG_STAGE_TIMES, UPTO_SCAN, &so); });
}

extern "C" int64_t gbwt_pfp_parse(void *storage, const uint8_t *T, int64_t n, int32_t W, int32_t P, uint32_t flags,
                                  int32_t *ranks, int32_t *parse_sa, int64_t capacity)
{
    Storage *st = (Storage *)storage;
    if (!st || !ranks || capacity < 1) return GBWT_BAD_PARAMETER;
    StageOut so;
    so.ranks = ranks;
    so.parse_sa = parse_sa;
    so.capacity = capacity;
    if (n == 0) return 0;
    return guarded([&]() { return pipeline(st, T, nullptr, n, W, P, flags & ~GBWT_FLAG_STAGE_TIMES, UPTO_PARSE, &so); });
}

extern "C" int64_t gbwt_set_kernel_probe(void *storage, int32_t kernel)
{
    Storage *st = (Storage *)storage;
    if (!st || kernel < -1 || kernel > GBWT_PROBE_SEG_SORT) return GBWT_BAD_PARAMETER;
    return guarded([&]() -> int64_t {
        if (kernel >= 0 && !st->probe_ev) {
            const int cap = 1024;
            st->probe_ev = (cudaEvent_t *)calloc(2 * cap, sizeof(cudaEvent_t));
            if (!st->probe_ev) return GBWT_NOT_ENOUGH_MEMORY;
            for (int i = 0; i < 2 * cap; i++) check_cuda(cudaEventCreate(&st->probe_ev[i]));
            st->probe_cap = cap;
        }
        check_cuda(cudaStreamSynchronize(st->stream));
        st->probe_kernel = kernel;
        st->probe_used = 0;
        st->probe_launches = 0;
        st->probe_bytes = 0;
        st->probe_ms = 0.0;
        return GBWT_NO_ERROR;
    });
}

// ---- libcubwt-compatible entry point ----------------------------------
namespace gbwt {

__global__ void k_byte_presence(const uint8_t *T, uint32_t n, uint32_t *bits)
{
    uint32_t m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t c = T[i];
#pragma unroll
        for (int w = 0; w < 8; w++) m[w] |= ((c >> 5) == (uint32_t)w) ? (1u << (c & 31u)) : 0u;
    }
#pragma unroll
    for (int w = 0; w < 8; w++) {
        const uint32_t v = __reduce_or_sync(0xFFFFFFFFu, m[w]);
        if ((threadIdx.x & 31u) == 0 && v) atomicOr(bits + w, v);
    }
}

// buf[i] = map[buf[i]]
__global__ void k_byte_map(uint8_t *buf, uint32_t n, const uint8_t *map)
{
    __shared__ uint8_t s_map[256];
    s_map[threadIdx.x] = map[threadIdx.x];      // blockDim == 256
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) buf[i] = s_map[buf[i]];
}

// libcubwt layout: L[0] = last, L[i] = O[i-1] for 1 <= i <= pidx, L[i] = O[i]
// after it (the reference convention's row pidx is libcubwt's '$' row).
__global__ void k_libcubwt_layout(const uint8_t *O, uint8_t *L, uint32_t n, uint32_t pidx, const uint8_t *unmap,
                                  uint8_t last)
{
    __shared__ uint8_t s_un[256];
    s_un[threadIdx.x] = unmap[threadIdx.x];      // blockDim == 256
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (i == 0) L[0] = last;
        else L[i] = s_un[i <= pidx ? O[i - 1] : O[i]];
    }
}

// libcubwt_bwt (r_log2 < 0) or libcubwt_bwt_aux (sampling rate 2^r_log2,
// I host array of (n-1) / 2^r_log2 + 1 entries).
static int64_t libcubwt_bwt(Storage *st, const uint8_t *T, uint8_t *L, int64_t n, int r_log2 = -1,
                            uint32_t *I = nullptr)
{
    const uint32_t un = (uint32_t)n;
    uint8_t *dT = slot<uint8_t>(st, S_TEXT, (size_t)n + 16);
    check_cuda(cudaMemcpyAsync(dT, T, (size_t)n, cudaMemcpyHostToDevice, st->stream));
    check_cuda(cudaMemsetAsync(st->d_flags + 8, 0, 8 * sizeof(uint32_t), st->stream));
    unsigned grid = grid_for(un, 256);
    if (grid > (unsigned)st->num_sms * 8) grid = (unsigned)st->num_sms * 8;
    k_byte_presence<<<grid, 256, 0, st->stream>>>(dT, un, st->d_flags + 8);
    after_launch(st);
    uint32_t present[8];
    check_cuda(cudaMemcpyAsync(st->h_scalars + 4, st->d_flags + 8, sizeof(present), cudaMemcpyDeviceToHost,
                               st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    memcpy(present, st->h_scalars + 4, sizeof(present));
    uint8_t *hmap = (uint8_t *)(st->h_scalars + 16);           // 256 pinned bytes each
    uint8_t *hunmap = (uint8_t *)(st->h_scalars + 48);
    uint32_t sigma = 0;
    bool identity = true;
    for (int c = 0; c < 256; c++) {
        hmap[c] = 0;
        hunmap[c] = (uint8_t)c;
    }
    for (int c = 0; c < 256; c++) {
        if ((present[c >> 5] >> (c & 31)) & 1u) {
            const uint32_t code = 2 + sigma++;
            if (code > 254) return GBWT_UNSUPPORTED_INPUT;      // 254..256 distinct values
            hmap[c] = (uint8_t)code;
            hunmap[code] = (uint8_t)c;
            if (c < 2 || c > 254) identity = false;
        }
    }
    uint8_t *dmaps = slot<uint8_t>(st, S_LCBMAP, 512);     // not touched by the pipeline
    if (!identity) {
        check_cuda(cudaMemcpyAsync(dmaps, hmap, 256, cudaMemcpyHostToDevice, st->stream));
        k_byte_map<<<grid, 256, 0, st->stream>>>(dT, un, dmaps);
        after_launch(st);
    } else {
        for (int c = 0; c < 256; c++) hunmap[c] = (uint8_t)c;
    }
    check_cuda(cudaMemcpyAsync(dmaps + 256, hunmap, 256, cudaMemcpyHostToDevice, st->stream));
    uint8_t *dO = slot<uint8_t>(st, S_OUT, (size_t)n + 16);
    uint32_t pidx;
    const size_t ni = r_log2 >= 0 ? (size_t)((n - 1) >> r_log2) + 1 : 0;
    uint32_t *dI = nullptr;
    if (r_log2 < 0) {
        int64_t rc = pipeline(st, dT, dO, n, 5, 16, GBWT_FLAG_DEVICE_POINTERS, UPTO_BWT, nullptr);
        if (rc < 0) return rc;
        pidx = (uint32_t)st->stats.primary_index;
    } else {
        // every suffix's row is needed at the sampled positions: the batched
        // path places all of them explicitly (one text)
        dI = slot<uint32_t>(st, S_GCHAR, ni);
        const int64_t offs[2] = {0, n};
        BatchAux aux;
        aux.r_log2 = r_log2;
        aux.dI = dI;
        int64_t rc = run_batch(st, dT, offs, 1, dO, 5, 16, GBWT_FLAG_DEVICE_POINTERS, MAX_N, &aux);
        if (rc < 0) return rc;
        check_cuda(cudaMemcpyAsync(I, dI, ni * 4, cudaMemcpyDeviceToHost, st->stream));
        check_cuda(cudaStreamSynchronize(st->stream));
        pidx = I[0] - 1u;                       // I[0] is the row of suffix 0, plus one
    }
    uint8_t *dL = slot<uint8_t>(st, S_LCB, (size_t)n + 16);
    k_libcubwt_layout<<<grid, 256, 0, st->stream>>>(dO, dL, un, pidx, dmaps + 256, T[n - 1]);
    after_launch(st);
    check_cuda(cudaMemcpyAsync(L, dL, (size_t)n, cudaMemcpyDeviceToHost, st->stream));
    check_cuda(cudaStreamSynchronize(st->stream));
    return (int64_t)pidx + 1;
}

}  // namespace gbwt

extern "C" int64_t gbwt_libcubwt_bwt(void *storage, const uint8_t *T, uint8_t *L, int64_t n)
{
    Storage *st = (Storage *)storage;
    if (!st || !T || !L || n < 1 || n > MAX_N) return GBWT_BAD_PARAMETER;
    return guarded([&]() { return libcubwt_bwt(st, T, L, n); });
}

extern "C" int64_t gbwt_libcubwt_bwt_aux(void *storage, const uint8_t *T, uint8_t *L, int64_t n, int64_t r,
                                         uint32_t *I)
{
    Storage *st = (Storage *)storage;
    if (!st || !T || !L || !I || n < 1 || n > MAX_N || r < 2 || (r & (r - 1)) != 0) return GBWT_BAD_PARAMETER;
    int r_log2 = 0;
    while ((1ll << r_log2) < r) r_log2++;
    return guarded([&]() -> int64_t {
        const int64_t rc = libcubwt_bwt(st, T, L, n, r_log2, I);
        return rc < 0 ? rc : GBWT_NO_ERROR;
    });
}

extern "C" int64_t gbwt_get_stats(void *storage, gbwt_stats *out)
{
    Storage *st = (Storage *)storage;
    if (!st || !out) return GBWT_BAD_PARAMETER;
    *out = st->stats;
    int64_t held = 0;
    for (int i = 0; i < S_NUM; i++) held += (int64_t)st->slots[i].cap;
    out->device_bytes = held;
    return GBWT_NO_ERROR;
}

extern "C" int64_t gbwt_check_tuning(const gbwt_tuning *t)
{
    if (!t) return GBWT_BAD_PARAMETER;
    const bool ok = (t->hash_log2_max == 0 || (t->hash_log2_max >= 16 && t->hash_log2_max <= 28)) &&
                    (t->batch_seg_tiles >= 0 && t->batch_seg_tiles <= 1024) &&
                    (t->batch_pad_eighths >= 0 && t->batch_pad_eighths <= 64) &&
                    (t->batch_radix_bits == 0 || t->batch_radix_bits == 8 || t->batch_radix_bits == 9) &&
                    (t->unbwt_rate_log2 == 0 || (t->unbwt_rate_log2 >= 2 && t->unbwt_rate_log2 <= 12)) &&
                    (t->dict_key_bits == 0 || (t->dict_key_bits >= 8 && t->dict_key_bits <= 64)) &&
                    (t->parse_key_phrases >= 0 && t->parse_key_phrases <= 2) &&
                    (t->mixed_radix_bits == 0 || t->mixed_radix_bits == 8 || t->mixed_radix_bits == 10) &&
                    (t->batch_ballot >= 0 && t->batch_ballot <= 3);
    return ok ? GBWT_NO_ERROR : GBWT_BAD_PARAMETER;
}

extern "C" int64_t gbwt_set_tuning(void *storage, const gbwt_tuning *t)
{
    Storage *st = (Storage *)storage;
    if (!st) return GBWT_BAD_PARAMETER;
    if (!t) {
        st->tuning = gbwt_tuning{};
        return GBWT_NO_ERROR;
    }
    const int64_t rc = gbwt_check_tuning(t);
    if (rc != GBWT_NO_ERROR) return rc;
    st->tuning = *t;
    return GBWT_NO_ERROR;
}

extern "C" int64_t gbwt_trim_device_storage(void *storage)
{
    Storage *st = (Storage *)storage;
    if (!st) return GBWT_BAD_PARAMETER;
    return guarded([&]() -> int64_t {
        check_cuda(cudaStreamSynchronize(st->stream));
        for (int i = 0; i < S_NUM; i++)
            if (st->slots[i].p) {
                check_cuda(cudaFree(st->slots[i].p));
                st->slots[i].p = nullptr;
                st->slots[i].cap = 0;
            }
        return GBWT_NO_ERROR;
    });
}

// ---- reference file formats (K:111-150, K:4776-4790) -----------------
extern "C" int64_t gbwt_read_input_txt(const char *path, uint8_t **T, int64_t *n)
{
    if (!path || !T || !n) return GBWT_BAD_PARAMETER;
    *T = nullptr;
    *n = 0;
    FILE *f = fopen(path, "rb");
    if (!f) return GBWT_BAD_PARAMETER;
    std::vector<char> buf;
    {
        char chunk[1 << 16];
        size_t r;
        while ((r = fread(chunk, 1, sizeof(chunk), f)) > 0) buf.insert(buf.end(), chunk, chunk + r);
    }
    fclose(f);
    buf.push_back('\0');
    const char *p = buf.data();
    auto skip = [&]() { while (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t') p++; };
    auto num = [&](int64_t &v) -> bool {
        skip();
        bool neg = false;
        if (*p == '-') { neg = true; p++; }
        if (*p < '0' || *p > '9') return false;
        v = 0;
        while (*p >= '0' && *p <= '9') {
            v = v * 10 + (*p - '0');
            if (v > (int64_t)1 << 40) return false;
            p++;
        }
        if (neg) v = -v;
        return true;
    };
    int64_t cnt;
    if (!num(cnt) || cnt < 0 || cnt > MAX_N) return GBWT_BAD_PARAMETER;
    uint8_t *out = (uint8_t *)malloc((size_t)cnt + 1);
    if (!out) return GBWT_NOT_ENOUGH_MEMORY;
    for (int64_t i = 0; i < cnt; i++) {
        int64_t v;
        if (!num(v) || v < 2 || v > 254) { free(out); return GBWT_BAD_PARAMETER; }
        out[i] = (uint8_t)v;
    }
    *T = out;
    *n = cnt;
    return cnt;
}

extern "C" int64_t gbwt_write_out_txt(const char *path, const uint8_t *L, int64_t n)
{
    if (!path || n < 0 || (n > 0 && !L)) return GBWT_BAD_PARAMETER;
    FILE *f = fopen(path, "wb");
    if (!f) return GBWT_BAD_PARAMETER;
    std::vector<char> buf;
    buf.reserve((size_t)n * 4 + 32);
    char tmp[32];
    int k = snprintf(tmp, sizeof(tmp), "%lld\n", (long long)n);
    buf.insert(buf.end(), tmp, tmp + k);
    for (int64_t i = 0; i < n; i++) {
        unsigned v = L[i];
        if (v >= 100) buf.push_back((char)('0' + v / 100));
        if (v >= 10) buf.push_back((char)('0' + (v / 10) % 10));
        buf.push_back((char)('0' + v % 10));
        buf.push_back(' ');
    }
    size_t w = fwrite(buf.data(), 1, buf.size(), f);
    int c = fclose(f);
    return (w == buf.size() && c == 0) ? n : GBWT_BAD_PARAMETER;
}

extern "C" void gbwt_free_host(void *p) { free(p); }

extern "C" const char *gbwt_error_string(int64_t code)
{
    switch (code) {
    case GBWT_NO_ERROR: return "no error";
    case GBWT_BAD_PARAMETER: return "bad parameter";
    case GBWT_NOT_ENOUGH_MEMORY: return "not enough host memory";
    case GBWT_GPU_ERROR: return "CUDA error";
    case GBWT_GPU_NOT_SUPPORTED: return "GPU not supported (library is built for sm_103a)";
    case GBWT_GPU_NOT_ENOUGH_MEMORY: return "not enough device memory";
    case GBWT_UNSUPPORTED_INPUT: return "input outside the variant's supported domain";
    case GBWT_TIMEOUT: return "device wait timed out";
    case GBWT_INTERNAL_ERROR: return "internal consistency check failed";
    default: return code >= 0 ? "no error" : "unknown error";
    }
}
