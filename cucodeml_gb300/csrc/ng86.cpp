// Pairwise Nei-Gojobori (1986) synonymous and nonsynonymous distances for
// clean codon data: the library's version of DistanceMatNG86
// (treesub.c:2270-2366) with difcodonNG (tools.c:305-420).
//
// codeml walks every pair of sequences over every pattern and re-derives the
// per-codon-pair counts (synonymous / nonsynonymous sites of both codons,
// synonymous / nonsynonymous differences averaged over the mutational paths
// that avoid stop codons) inside that double loop.  Those counts depend only
// on the two sense codons, so here they are tabulated once for the 61 x 61
// pairs; a sequence pair is then five weighted sums over the patterns, and the
// pairs are split over host threads.  Host setup work (no device involved).
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "gbcodeml.h"

namespace {

const char kAA64[] = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG";

struct PairCounts {
    double sites_syn, sites_non;   // S and N of the two codons together
    double diff_syn, diff_non;     // path-averaged synonymous / nonsynonymous differences
};

// the amino acid of a 64-codon index (TCAG order, 16 b0 + 4 b1 + b2), '*' for a stop
inline char aa_of(int c) { return kAA64[c]; }

// synonymous neighbours and stop neighbours of one codon over its 9 single-base changes
void neighbours(int c, int &syn, int &stop) {
    const int by[3] = {16, 4, 1};
    syn = stop = 0;
    for (int j = 0; j < 3; j++) {
        const int b = (c / by[j]) % 4;
        for (int k = 0; k < 4; k++) {
            if (k == b) continue;
            const char a = aa_of(c + (k - b) * by[j]);
            if (a == '*') stop++;
            else if (a == aa_of(c)) syn++;
        }
    }
}

// differences between codons from (c0) and to (c1): ndiff, and syn / non
// averaged over the orders of the differing positions whose intermediate
// codons are not stops (all paths through stops: codeml's fixed fallback)
int differences(int c0, int c1, double &ds, double &dn) {
    const int by[3] = {16, 4, 1};
    int b0[3], b1[3], mark[3], nd = 0;
    for (int j = 0; j < 3; j++) {
        b0[j] = (c0 / by[j]) % 4;
        b1[j] = (c1 / by[j]) % 4;
        if (b0[j] != b1[j]) mark[nd++] = j;
    }
    ds = dn = 0;
    if (nd == 0) return 0;
    if (nd == 1) {
        (aa_of(c0) == aa_of(c1) ? ds : dn) += 1;
        return 1;
    }
    const int npath = nd == 2 ? 2 : 6;
    int nstop = 0;
    for (int p = 0; p < npath; p++) {
        int order[3];
        if (nd == 2) {
            order[0] = mark[p];
            order[1] = mark[1 - p];
        } else {   // the 6 orders of positions 0, 1, 2
            order[0] = p / 2;
            order[1] = p % 2;
            if (order[0] <= order[1]) order[1]++;
            order[2] = 3 - order[0] - order[1];
        }
        int cur[3] = {b0[0], b0[1], b0[2]};
        int s = 0, n = 0;
        bool blocked = false;
        for (int st = 0; st < nd; st++) {
            const int from = 16 * cur[0] + 4 * cur[1] + cur[2];
            cur[order[st]] = b1[order[st]];
            const int to = 16 * cur[0] + 4 * cur[1] + cur[2];
            if (aa_of(to) == '*') {
                blocked = true;
                break;
            }
            (aa_of(from) == aa_of(to) ? s : n)++;
        }
        if (blocked) {
            nstop++;
            continue;
        }
        ds += s;
        dn += n;
    }
    if (nstop == npath) {
        ds = nd == 2 ? 0 : 1;
        dn = 2;
    } else {
        ds /= npath - nstop;
        dn /= npath - nstop;
    }
    return nd;
}

}  // namespace

extern "C" int gb_ng86(int ns, int npatt, const unsigned char *z, const double *fpatt, double *dS, double *dN,
                       double *dist) {
    if (ns < 2 || npatt < 1 || !z || !fpatt || !dS || !dN) return GB_ERR_ARG;
    for (size_t i = 0; i < (size_t)ns * npatt; i++)
        if (z[i] >= GB_NCODE) return GB_ERR_ARG;
    int sense[61], n = 0;
    for (int i = 0; i < 64; i++)
        if (kAA64[i] != '*') sense[n++] = i;
    int syn[61], stop[61];
    for (int c = 0; c < 61; c++) neighbours(sense[c], syn[c], stop[c]);
    std::vector<PairCounts> tab(61 * 61);
    for (int a = 0; a < 61; a++)
        for (int b = 0; b < 61; b++) {
            PairCounts &t = tab[a * 61 + b];
            t.sites_syn = (syn[a] + syn[b]) * (3 / 18.);
            t.sites_non = 3 * (1 - (stop[a] + stop[b]) / 18.) - t.sites_syn;
            differences(sense[b], sense[a], t.diff_syn, t.diff_non);
        }
    const double bigD = 3;
    auto one_pair = [&](int is, int js) {
        double lst = 0, S = 0, N = 0, nst = 0, nat = 0;
        const unsigned char *zi = z + (size_t)is * npatt, *zj = z + (size_t)js * npatt;
        for (int h = 0; h < npatt; h++) {
            const PairCounts &t = tab[zi[h] * 61 + zj[h]];
            const double w = fpatt[h];
            lst += w;
            S += t.sites_syn * w;
            N += t.sites_non * w;
            nst += t.diff_syn * w;
            nat += t.diff_non * w;
        }
        if (S > 0 && N > 0) {   // rescale for stop codons
            const double y = lst * 3. / (S + N);
            S *= y;
            N *= y;
        }
        double ps = S <= 0 ? 0 : 1 - 4. / 3 * nst / S;
        double pn = N <= 0 ? 0 : 1 - 4. / 3 * nat / N;
        double vs = ps == 1 ? 0 : (ps <= 0 ? -1 : 3. / 4 * (-std::log(ps)));
        double vn = pn == 1 ? 0 : (pn <= 0 ? -1 : 3. / 4 * (-std::log(pn)));
        dS[is * ns + js] = dS[js * ns + is] = vs;
        dN[is * ns + js] = dN[js * ns + is] = vn;
        if (dist) {
            if (N > 0 && vn < 0) vn = bigD;
            if (S > 0 && vs < 0) vs = bigD;
            dist[is * ns + js] = dist[js * ns + is] = (S <= 0 || N <= 0) ? 0 : (S * vs + N * vn) * 3 / (S + N);
        }
    };
    for (int i = 0; i < ns; i++) {
        dS[i * ns + i] = dN[i * ns + i] = 0;
        if (dist) dist[i * ns + i] = 0;
    }
    const long npair = (long)ns * (ns - 1) / 2;
    const int nth = (int)std::max(1L, std::min<long>(std::thread::hardware_concurrency(), npair / 64 + 1));
    std::vector<std::thread> pool;
    for (int t = 0; t < nth; t++)
        pool.emplace_back([&, t]() {
            for (long p = t; p < npair; p += nth) {
                // pair p = is (is - 1) / 2 + js with js < is
                int is = (int)((1 + std::sqrt(1.0 + 8.0 * p)) / 2);
                while ((long)is * (is - 1) / 2 > p) is--;
                while ((long)(is + 1) * is / 2 <= p) is++;
                one_pair(is, (int)(p - (long)is * (is - 1) / 2));
            }
        });
    for (auto &th : pool) th.join();
    return GB_OK;
}
