// Codon site-pattern compression and F3x4 codon frequencies for clean codon
// data: the library's own version of PatternWeight + EncodeSeqs
// (treesub.c:1075-1143, 1302-1439) and CountCodons / Fcodon_3x4 /
// InitializeCodon (codeml.c:3475-3570, 3732-3742).
//
// codeml keeps the unique sites sorted by strcmp of their nucleotide letters
// (species-major, three letters per codon, each letter + 1), so pattern h is
// the h-th distinct site in that order and fpatt[h] counts its sites.  Letters
// compare by ASCII (A < C < G < T), which is the order used here via ranks.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "gbcodeml.h"

namespace {
const char kAA64[] = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG";
}

extern "C" int gb_patterns(int ns, int ncodon, const int *codons, int *npatt_out, unsigned char *z,
                           double *fpatt, double *pi) {
    if (ns < 1 || ncodon < 1 || !codons || !npatt_out || !z || !fpatt || !pi) return GB_ERR_ARG;
    int sense[61], n = 0;
    for (int i = 0; i < 64; i++)
        if (kAA64[i] != '*') sense[n++] = i;
    // letter ranks in ASCII order for bases indexed T, C, A, G
    const unsigned char rank[4] = {3, 1, 0, 2};
    const int L = 3 * ns;
    std::vector<unsigned char> key((size_t)ncodon * L);
    for (int h = 0; h < ncodon; h++)
        for (int j = 0; j < ns; j++) {
            int c = codons[(size_t)j * ncodon + h];
            if (c < 0 || c >= 61) return GB_ERR_ARG;
            int ic = sense[c];
            unsigned char *k = &key[(size_t)h * L + 3 * j];
            k[0] = rank[ic / 16];
            k[1] = rank[(ic / 4) % 4];
            k[2] = rank[ic % 4];
        }
    std::vector<int> idx(ncodon);
    std::iota(idx.begin(), idx.end(), 0);
    auto K = [&](int h) { return &key[(size_t)h * L]; };
    std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return std::memcmp(K(a), K(b), L) < 0; });
    std::vector<int> first;   // representative site per pattern
    std::vector<double> cnt;
    for (int s = 0; s < ncodon; s++) {
        if (s == 0 || std::memcmp(K(idx[s]), K(idx[s - 1]), L) != 0) {
            first.push_back(idx[s]);
            cnt.push_back(0.0);
        }
        cnt.back() += 1.0;
    }
    const int np = (int)first.size();
    for (int j = 0; j < ns; j++)
        for (int h = 0; h < np; h++) z[(size_t)j * np + h] = (unsigned char)codons[(size_t)j * ncodon + first[h]];
    for (int h = 0; h < np; h++) fpatt[h] = cnt[h];
    *npatt_out = np;
    // F3x4: codon counts over species and patterns, base frequencies by
    // codon position, product over the sense codons, normalised
    double fcodon[64] = {0}, fb[12] = {0};
    for (int j = 0; j < ns; j++)
        for (int h = 0; h < np; h++) fcodon[sense[z[(size_t)j * np + h]]] += fpatt[h];
    for (int k = 0; k < 64; k++) {
        fb[0 + k / 16] += fcodon[k];
        fb[4 + (k % 16) / 4] += fcodon[k];
        fb[8 + k % 4] += fcodon[k];
    }
    for (int j = 0; j < 3; j++) {
        double t = fb[j * 4] + fb[j * 4 + 1] + fb[j * 4 + 2] + fb[j * 4 + 3];
        if (!(t > 0)) return GB_ERR_ARG;
        t = 1 / t;
        for (int b = 0; b < 4; b++) fb[j * 4 + b] *= t;
    }
    double s = 0;
    for (int c = 0; c < 61; c++) {
        int k = sense[c];
        pi[c] = fb[k / 16] * fb[4 + (k / 4) % 4] * fb[8 + k % 4];
    }
    for (int c = 0; c < 61; c++) s += pi[c];
    s = 1 / s;
    for (int c = 0; c < 61; c++) pi[c] *= s;
    return GB_OK;
}
