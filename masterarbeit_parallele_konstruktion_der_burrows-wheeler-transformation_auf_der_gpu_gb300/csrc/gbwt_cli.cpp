// gbwt_cli.cpp -- command-line drop-in for the reference's PFP programs.
//
// The reference builds one binary per (W, P, small-alphabet) variant
// (Makefile:11-23, e.g. Prefix_Free_Parsing_W=5_P=16_Linux); each reads
// ./input.txt and writes ./out.txt (K:111-150, K:4776-4790 of
// Prefix_Free_Parsing_W=5_P=16_kommentiert.cu) and takes no arguments.
// This program does the same.  The variant comes from the name it is run
// under (a symlink named like a reference binary) or from
// --W/--P/--small; --in/--out change the file names.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <string>
#include "../../include/gbwt.h"

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

int main(int argc, char **argv)
{
    int W = 5, P = 16;
    bool small = false;
    std::string in = "input.txt", out = "out.txt";
    std::string bin_in, bin_out;          // raw-byte fast path instead of decimal text
    std::string self = argv[0];
    size_t slash = self.find_last_of('/');
    if (slash != std::string::npos) self = self.substr(slash + 1);
    parse_variant(self, W, P, small);
    for (int i = 1; i < argc; i++) {
        std::string a = argv[i];
        if (a == "--W" && i + 1 < argc) W = atoi(argv[++i]);
        else if (a == "--P" && i + 1 < argc) P = atoi(argv[++i]);
        else if (a == "--small") small = true;
        else if (a == "--in" && i + 1 < argc) in = argv[++i];
        else if (a == "--out" && i + 1 < argc) out = argv[++i];
        else if (a == "--binary-in" && i + 1 < argc) bin_in = argv[++i];
        else if (a == "--binary-out" && i + 1 < argc) bin_out = argv[++i];
        else if (a == "--variant" && i + 1 < argc) {
            if (!parse_variant(argv[++i], W, P, small)) { fprintf(stderr, "bad variant name\n"); return 2; }
        } else {
            fprintf(stderr, "usage: %s [--W w --P p --small] [--variant NAME] [--in input.txt] [--out out.txt]"
                            " [--binary-in FILE] [--binary-out FILE]\n",
                    argv[0]);
            return 2;
        }
    }
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
