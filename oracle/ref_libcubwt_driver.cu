/*
 * ref_libcubwt_driver.cu -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * Timing driver around the libcubwt 1.6.3 copy that the reference ships
 * (libcubwt.cu / libcubwt.cuh), compiled UNMODIFIED: libcubwt.cu is included
 * with its harness `main` (libcubwt.cu:3023-3037) renamed.  What this file
 * replaces is that harness's decimal `input.txt` reader and its `out.txt`
 * printer; the output is re-assembled exactly as its print_Output does
 * (libcubwt.cu:2989-3020): with primary index p, the bytes are
 * L[1..p-1], L[0], L[p..n-1] -- the convention the reference's
 * compare_script.sh `cmp`s the PFP output against.
 *
 * Usage: ref_libcubwt <text.bin> <bwt.bin> [repetitions]
 * The device storage is allocated once, outside the timed calls
 * (libcubwt_allocate_device_storage, libcubwt.cuh:60); one untimed warm-up
 * call, then `repetitions` timed calls of libcubwt_bwt (libcubwt.cu:2414-2431)
 * on pinned host buffers.  libcubwt_bwt copies the text in and the BWT out
 * inside the call, so every time is the host-to-host span.  Prints one JSON
 * line with the median and every time.
 */
#define main gbo_libcubwt_program_main
#include "libcubwt.cu"
#undef main

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

int main(int argc, char** argv)
{
    if (argc < 3) {
        fprintf(stderr, "usage: %s <text.bin> <bwt.bin> [repetitions]\n", argv[0]);
        return 2;
    }
    int reps = argc > 3 ? atoi(argv[3]) : 1;
    if (reps < 1) reps = 1;
    FILE* f = fopen(argv[1], "rb");
    if (!f) { fprintf(stderr, "cannot read %s\n", argv[1]); return 2; }
    fseek(f, 0, SEEK_END);
    long len = ftell(f);
    fseek(f, 0, SEEK_SET);
    if (len < 16) { fprintf(stderr, "libcubwt needs at least 16 bytes\n"); fclose(f); return 3; }
    uint8_t* T = nullptr;
    uint8_t* L = nullptr;
    if (cudaMallocHost((void**)&T, (size_t)len) != cudaSuccess ||
        cudaMallocHost((void**)&L, (size_t)len) != cudaSuccess) {
        fprintf(stderr, "pinned host allocation failed\n");
        return 4;
    }
    if (fread(T, 1, (size_t)len, f) != (size_t)len) { fprintf(stderr, "short read\n"); return 2; }
    fclose(f);

    void* storage = nullptr;
    int64_t rc = libcubwt_allocate_device_storage(&storage, (int64_t)len);
    if (rc != LIBCUBWT_NO_ERROR) { fprintf(stderr, "libcubwt_allocate_device_storage: %lld\n", (long long)rc); return 4; }

    int64_t index = libcubwt_bwt(storage, T, L, (int64_t)len); /* warm-up */
    std::vector<double> ms;
    for (int r = 0; r < reps && index > 0; r++) {
        auto t0 = std::chrono::steady_clock::now();
        index = libcubwt_bwt(storage, T, L, (int64_t)len);
        auto t1 = std::chrono::steady_clock::now();
        ms.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
    }
    libcubwt_free_device_storage(storage);
    if (index <= 0) { fprintf(stderr, "libcubwt_bwt: %lld\n", (long long)index); return 4; }

    /* print_Output(index), libcubwt.cu:2989-3020, in raw bytes */
    f = fopen(argv[2], "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", argv[2]); return 2; }
    size_t p = (size_t)index;
    bool ok = fwrite(L + 1, 1, p - 1, f) == p - 1 && fwrite(L, 1, 1, f) == 1 &&
              fwrite(L + p, 1, (size_t)len - p, f) == (size_t)len - p;
    fclose(f);
    if (!ok) { fprintf(stderr, "short write\n"); return 2; }

    std::vector<double> sorted = ms;
    std::sort(sorted.begin(), sorted.end());
    printf("{\"n\": %ld, \"primary_index\": %lld, \"host_ms\": %.4f, \"host_ms_all\": [", len, (long long)index,
           sorted[sorted.size() / 2]);
    for (size_t i = 0; i < ms.size(); i++) printf("%s%.4f", i ? ", " : "", ms[i]);
    printf("]}\n");
    cudaFreeHost(T);
    cudaFreeHost(L);
    return 0;
}
