// gbwt_cli.cpp -- command-line drop-in for the reference's BWT programs.
//
// The reference builds one binary per (W, P, small-alphabet) PFP variant
// (Makefile:11-23, e.g. Prefix_Free_Parsing_W=5_P=16_Linux), plus
// Lyndon_Grammar_BWT_Linux and libcubwt_Linux (Makefile:21-22); each reads
// ./input.txt and writes ./out.txt (K:111-150, K:4776-4790 of
// Prefix_Free_Parsing_W=5_P=16_kommentiert.cu; LY:365-402, LY:5530-5545 of
// Lyndon_Grammar_BWT.cu; LC:2971-3037 of libcubwt.cu) and takes no arguments.
// This program does the same.  The program comes from the name it is run
// under (a symlink named like a reference binary) or from
// --W/--P/--small/--libcubwt; --in/--out change the file names.
//
//  * PFP names: the PFP BWT with that W, P and alphabet.
//  * Lyndon_Grammar_BWT: the same BWT (the reference checks its output
//    against libcubwt's with cmp, compare_script_lyndon.sh), built here by
//    the PFP pipeline with W=5, P=16; the same input range (bytes 2..254,
//    LY:388).
//  * libcubwt: any byte values; gbwt_libcubwt_bwt, written the way the
//    libcubwt harness writes (LC:2989-3020): the raw layout when the
//    returned index is 0, else the layout with L[0] moved to the index
//    (nothing is written for L[0] when the index is n, as there).
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <string>
#include <vector>
#include "../../include/gbwt.h"

enum class Program { pfp, libcubwt };

static bool parse_variant(const std::string &name, int &W, int &P, bool &small)
{
    // Prefix_Free_Parsing_W=<W>_P=<P>[_small_alphabet][_Linux]
    size_t w = name.find("W="), p = name.find("_P=");
    if (w == std::string::npos || p == std::string::npos) return false;
    W = atoi(name.c_str() + w + 2);
    P = atoi(name.c_str() + p + 3);
    small = name.find("small_alphabet") != std::string::npos;
    return W > 0 && P > 0;
}

// The program a reference binary name stands for.
static Program program_of(const std::string &name, int &W, int &P, bool &small)
{
    if (name.compare(0, 8, "libcubwt") == 0) return Program::libcubwt;
    if (name.compare(0, 18, "Lyndon_Grammar_BWT") == 0) {
        W = 5;
        P = 16;
        small = false;
        return Program::pfp;
    }
    parse_variant(name, W, P, small);
    return Program::pfp;
}

// input.txt with any byte values (libcubwt's harness reads every value into
// a byte, LC:2971-2985); values outside 0..255 are an error here.
static int64_t read_any_bytes(const char *path, std::vector<uint8_t> &T)
{
    FILE *f = fopen(path, "rb");
    if (!f) return GBWT_BAD_PARAMETER;
    long long cnt;
    if (fscanf(f, "%lld", &cnt) != 1 || cnt < 0 || cnt > (1ll << 31) - 2) { fclose(f); return GBWT_BAD_PARAMETER; }
    T.resize((size_t)cnt);
    for (long long i = 0; i < cnt; i++) {
        int v;
        if (fscanf(f, "%d", &v) != 1 || v < 0 || v > 255) { fclose(f); return GBWT_BAD_PARAMETER; }
        T[(size_t)i] = (uint8_t)v;
    }
    fclose(f);
    return cnt;
}

static int run_libcubwt(const std::string &in, const std::string &out)
{
    std::vector<uint8_t> T;
    int64_t rc = read_any_bytes(in.c_str(), T);
    if (rc < 0) { fprintf(stderr, "gbwt_pfp: cannot read %s\n", in.c_str()); return 1; }
    const int64_t n = (int64_t)T.size();
    std::vector<uint8_t> L((size_t)n + 1);
    void *st = nullptr;
    rc = gbwt_allocate_device_storage(&st, n);
    if (rc < 0) { fprintf(stderr, "gbwt_pfp: %s\n", gbwt_error_string(rc)); return 1; }
    const int64_t index = gbwt_libcubwt_bwt(st, T.data(), L.data(), n);
    gbwt_free_device_storage(st);
    if (index < 0) { fprintf(stderr, "gbwt_pfp: %s\n", gbwt_error_string(index)); return 1; }
    FILE *f = fopen(out.c_str(), "wb");
    if (!f) { fprintf(stderr, "gbwt_pfp: cannot write %s\n", out.c_str()); return 1; }
    fprintf(f, "%lld\n", (long long)n);
    if (index == 0) {
        for (int64_t i = 0; i < n; i++) fprintf(f, "%d ", L[(size_t)i]);
    } else {
        for (int64_t i = 1; i < n; i++) {
            if (i == index) fprintf(f, "%d ", L[0]);
            fprintf(f, "%d ", L[(size_t)i]);
        }
    }
    const bool ok = fclose(f) == 0;
    if (!ok) { fprintf(stderr, "gbwt_pfp: cannot write %s\n", out.c_str()); return 1; }
    return 0;
}

int main(int argc, char **argv)
{
    int W = 5, P = 16;
    bool small = false;
    std::string in = "input.txt", out = "out.txt";
    std::string bin_in, bin_out;          // raw-byte fast path instead of decimal text
    std::string self = argv[0];
    size_t slash = self.find_last_of('/');
    if (slash != std::string::npos) self = self.substr(slash + 1);
    Program prog = program_of(self, W, P, small);
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a == "--libcubwt") prog = Program::libcubwt;
        else if (a == "--W" && i + 1 < argc) W = atoi(argv[++i]);
        else if (a == "--P" && i + 1 < argc) P = atoi(argv[++i]);
        else if (a == "--small") small = true;
        else if (a == "--in" && i + 1 < argc) in = argv[++i];
        else if (a == "--out" && i + 1 < argc) out = argv[++i];
        else if (a == "--binary-in" && i + 1 < argc) bin_in = argv[++i];
        else if (a == "--binary-out" && i + 1 < argc) bin_out = argv[++i];
        else if (a == "--variant" && i + 1 < argc) {
            if (!parse_variant(argv[++i], W, P, small)) { fprintf(stderr, "bad variant name\n"); return 2; }
        } else {
            fprintf(stderr, "usage: %s [--W w --P p --small | --libcubwt] [--variant NAME] [--in input.txt]"
                            " [--out out.txt] [--binary-in FILE] [--binary-out FILE]\n",
                    argv[0]);
            return 2;
        }
    }
    if (prog == Program::libcubwt) return run_libcubwt(in, out);
    uint8_t *T = nullptr;
    int64_t n = 0;
    int64_t rc;
    if (!bin_in.empty()) {
        // raw bytes: no decimal parsing (the reference's fscanf loop dominates
        // its wall time on large inputs, K:111-150)
        FILE *f = fopen(bin_in.c_str(), "rb");
        if (!f) { fprintf(stderr, "gbwt_pfp: cannot open %s\n", bin_in.c_str()); return 1; }
        fseek(f, 0, SEEK_END);
        long sz = ftell(f);
        fseek(f, 0, SEEK_SET);
        T = (uint8_t *)malloc(sz > 0 ? (size_t)sz : 1);
        n = (int64_t)fread(T, 1, sz > 0 ? (size_t)sz : 0, f);
        fclose(f);
        rc = n;
    } else {
        rc = gbwt_read_input_txt(in.c_str(), &T, &n);
    }
    if (rc < 0) { fprintf(stderr, "gbwt_pfp: cannot read %s: %s\n", in.c_str(), gbwt_error_string(rc)); return 1; }
    void *st = nullptr;
    rc = gbwt_allocate_device_storage(&st, n);
    if (rc < 0) { fprintf(stderr, "gbwt_pfp: %s\n", gbwt_error_string(rc)); gbwt_free_host(T); return 1; }
    uint8_t *L = (uint8_t *)malloc((size_t)n + 1);
    rc = gbwt_pfp_bwt(st, T, L, n, W, P, small ? GBWT_FLAG_SMALL_ALPHABET : 0u);
    if (rc < 0) {
        fprintf(stderr, "gbwt_pfp: %s\n", gbwt_error_string(rc));
        gbwt_free_device_storage(st);
        gbwt_free_host(T);
        free(L);
        return 1;
    }
    if (!bin_out.empty()) {
        FILE *f = fopen(bin_out.c_str(), "wb");
        rc = (f && fwrite(L, 1, (size_t)n, f) == (size_t)n) ? n : -1;
        if (f) fclose(f);
    } else {
        rc = gbwt_write_out_txt(out.c_str(), L, n);
    }
    gbwt_free_device_storage(st);
    gbwt_free_host(T);
    free(L);
    if (rc < 0) { fprintf(stderr, "gbwt_pfp: cannot write %s\n", out.c_str()); return 1; }
    return 0;
}
