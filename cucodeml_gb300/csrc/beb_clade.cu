// The grid integral of codeml's Bayes empirical Bayes analysis under the
// clade models C and D with two branch types, on the device
// (lfunNSsites_ACD codeml.c:6617-6826 with modelACD = mC / mD; grid and
// omega sets get_grid_para_like_ACD 6419-6530).
//
// Input: log f(x_h | w) of every omega set (gb_beb_tables computes them on the
// device from the handle's forward; the caller hands them back in set order):
//   clade C, 111 sets: 0..9  w0_i (grid in (0, 1)) on every branch,
//                      10    w = 1 on every branch,
//                      11 + 10 i + j  w2_i background, w3_j foreground;
//   clade D, 120 sets: 0..9  w0_i (grid in (0, 0.5)), 10..19  w1_i (grid in
//                      (0.5, 1.5)) on every branch, 20 + 10 i + j as above;
//   w2, w3 on a grid in (0, 3).
// Grid: 100 ternary (p0, p1) triangles x w0 x (D: w1) x w2 x w3 (10^5 points
// for C, 10^6 for D), uniform.  At grid point g the three classes have
// proportions (p0, p1, p2) of its triangle and f(x_h | g) = sum_c p_c F_c(g)[h].
//
// 1. per pattern: the maximum over the sets (codeml's S1) and F = exp(L - max);
// 2. lnfXs[g] = sum_h fpatt_h log f(x_h | g): one block per grid point,
//    threads over patterns (coalesced rows of F);
// 3. the marginal log f(X) with codeml's running scale S2, the grid and
//    (p0, p1) marginals: a sequential loop on the host, as for model A;
// 4. posteriors post[c][h] = sum_g w_g p_c F_c(g)[h] / f(x_h | g), w_g =
//    exp(lnfXs[g] - log f(X)), terms above exp(-300) as codeml adds them: one
//    warp per pattern, lanes over the grid, the pattern's sets in shared memory.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <algorithm>
#include <vector>

#include "gbcodeml.h"
#include "handle.h"

namespace gb {
namespace {

constexpr int CD = GB_BEB_GRID;          // grid points per dimension (10)
constexpr int CNT = CD * CD;             // (p0, p1) triangles
constexpr int CNK = CD * CD;             // (w2, w3) pairs
constexpr int CMAXW = 2 * CD + CNK;      // sets of clade D (the larger)

struct CladeGrid {
    int n1;        // w1 values (1 for C: the single set w = 1)
    int b1, b2;    // first set of class 1 and of class 2
    int nsets, ngrid;
};

__host__ __device__ inline CladeGrid clade_grid(int model_d) {
    CladeGrid c;
    c.n1 = model_d ? CD : 1;
    c.b1 = CD;
    c.b2 = CD + c.n1;
    c.nsets = c.b2 + CNK;
    c.ngrid = CNT * CD * c.n1 * CNK;
    return c;
}

// g = ((t CD + i0) n1 + i1) CNK + k
__device__ __forceinline__ void clade_sets(const CladeGrid &c, int g, int &t, int &s0, int &s1, int &s2) {
    const int k = g % CNK;
    int q = g / CNK;
    const int i1 = q % c.n1;
    q /= c.n1;
    const int i0 = q % CD;
    t = q / CD;
    s0 = i0;
    s1 = c.b1 + i1;
    s2 = c.b2 + k;
}

__global__ void __launch_bounds__(256) clade_rescale_kernel(const double *__restrict__ L, double *__restrict__ F,
                                                            double *__restrict__ mrow, int nsets, int npatt) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= npatt) return;
    double m = L[h];
    for (int s = 1; s < nsets; s++) m = fmax(m, L[(size_t)s * npatt + h]);
    for (int s = 0; s < nsets; s++) F[(size_t)s * npatt + h] = exp(L[(size_t)s * npatt + h] - m);
    mrow[h] = m;
}

__global__ void __launch_bounds__(256) clade_grid_kernel(CladeGrid c, const double *__restrict__ F,
                                                         const double *__restrict__ fpatt,
                                                         const double *__restrict__ ptri, int npatt,
                                                         double *__restrict__ lnfXs) {
    __shared__ double red[8];
    const int g = blockIdx.x;
    int t, s0, s1, s2;
    clade_sets(c, g, t, s0, s1, s2);
    const double p0 = ptri[3 * t], p1 = ptri[3 * t + 1], p2 = ptri[3 * t + 2];
    const double *r0 = F + (size_t)s0 * npatt, *r1 = F + (size_t)s1 * npatt, *r2 = F + (size_t)s2 * npatt;
    double s = 0.0;
    for (int h = threadIdx.x; h < npatt; h += blockDim.x) {
        double fh = p0 * r0[h];
        fh += p1 * r1[h];
        fh += p2 * r2[h];
        if (fh < 1e-300) continue;
        s += log(fh) * fpatt[h];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) v += red[w];
        lnfXs[g] = v;
    }
}

// wt[g] = (w_g, exp(-300) / w_g): a term ratio * w_g is added when ratio > the second
__global__ void __launch_bounds__(256) clade_post_kernel(CladeGrid c, const double *__restrict__ F,
                                                         const double *__restrict__ ptri,
                                                         const double2 *__restrict__ wt, int npatt,
                                                         double *__restrict__ post) {
    __shared__ double fs[8][CMAXW + 4];
    __shared__ double ps[CNT * 3];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < CNT * 3; i += blockDim.x) ps[i] = ptri[i];
    const int h = blockIdx.x * 8 + warp;
    if (h < npatt)
        for (int s = lane; s < c.nsets; s += 32) fs[warp][s] = F[(size_t)s * npatt + h];
    __syncthreads();
    if (h >= npatt) return;
    const double *f = fs[warp];
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int g = lane; g < c.ngrid; g += 32) {
        int t, s0, s1, s2;
        clade_sets(c, g, t, s0, s1, s2);
        const double2 w = wt[g];
        const double f0 = ps[3 * t] * f[s0], f1 = ps[3 * t + 1] * f[s1], f2 = ps[3 * t + 2] * f[s2];
        const double tot = (f0 + f1) + f2;
        if (!(tot > 0.0)) continue;
        const double inv = 1.0 / tot;
        double r = f0 * inv;
        if (r > w.y) a0 += r * w.x;
        r = f1 * inv;
        if (r > w.y) a1 += r * w.x;
        r = f2 * inv;
        if (r > w.y) a2 += r * w.x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, o);
        a1 += __shfl_down_sync(0xffffffffu, a1, o);
        a2 += __shfl_down_sync(0xffffffffu, a2, o);
    }
    if (lane == 0) {
        post[h] = a0;
        post[(size_t)npatt + h] = a1;
        post[(size_t)2 * npatt + h] = a2;
    }
}

// (p0, p1, p2) at the centroids of the 100 ternary triangles (GetIndexTernary tools.c:4441-4461)
void ternary(double *ptri) {
    for (int t = 0; t < CNT; t++) {
        const int ix = (int)std::floor(std::sqrt((double)t)), iy = t - ix * ix;
        const double a = (1 + (iy / 2) * 3 + (iy % 2)) / (3.0 * CD);
        const double b = (1 + (CD - 1 - ix) * 3 + (iy % 2)) / (3.0 * CD);
        ptri[3 * t] = a;
        ptri[3 * t + 1] = b;
        ptri[3 * t + 2] = 1 - a - b;
    }
}

struct CladeBuffers {
    double *L = nullptr, *F = nullptr, *mrow = nullptr, *ptri = nullptr, *lnfXs = nullptr, *post = nullptr;
    double2 *wt = nullptr;
    ~CladeBuffers() {
        void *p[] = {L, F, mrow, ptri, lnfXs, post, wt};
        for (void *q : p)
            if (q) cudaFree(q);
    }
};

}  // namespace
}  // namespace gb

int gb_beb_clade(gb_handle *h, int model_d, const double *lnfw, double *post_out, double *grid_out,
                 double *p0p1_out, double *lnfX_out, gb_stats *stats) {
    using namespace gb;
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!lnfw || (model_d != 0 && model_d != 1)) return fail(GB_ERR_ARG, "gb_beb_clade: bad arguments");
    const CladeGrid c = clade_grid(model_d);
    const int npatt = h->npatt;
    const double t0 = now_ms();
    CK(cudaSetDevice(h->device));
    cudaStream_t st = h->stream;
    CladeBuffers B;
    int rc;
    if ((rc = dalloc(&B.L, (size_t)c.nsets * npatt)) || (rc = dalloc(&B.F, (size_t)c.nsets * npatt)) ||
        (rc = dalloc(&B.mrow, npatt)) || (rc = dalloc(&B.ptri, 3 * CNT)) || (rc = dalloc(&B.lnfXs, c.ngrid)) ||
        (rc = dalloc(&B.post, (size_t)3 * npatt)) || (rc = dalloc(&B.wt, c.ngrid)))
        return rc;
    std::vector<double> ptri(3 * CNT);
    ternary(ptri.data());
    CK(cudaEventRecord(h->ev0, st));
    CK(cudaMemcpyAsync(B.L, lnfw, sizeof(double) * c.nsets * npatt, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B.ptri, ptri.data(), sizeof(double) * 3 * CNT, cudaMemcpyHostToDevice, st));
    clade_rescale_kernel<<<(npatt + 255) / 256, 256, 0, st>>>(B.L, B.F, B.mrow, c.nsets, npatt);
    clade_grid_kernel<<<c.ngrid, 256, 0, st>>>(c, B.F, h->d_fpatt, B.ptri, npatt, B.lnfXs);
    CK(cudaGetLastError());
    std::vector<double> mrow(npatt), lnfXs(c.ngrid);
    CK(cudaMemcpyAsync(mrow.data(), B.mrow, sizeof(double) * npatt, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(lnfXs.data(), B.lnfXs, sizeof(double) * c.ngrid, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    // S1, then the marginal over the grid with codeml's running scale S2
    // (codeml.c:6700-6747): a new largest term rescales the sums so far
    double S1 = 0;
    for (int q = 0; q < npatt; q++) S1 += mrow[q] * h->fpatt[q];
    std::vector<double> pp((size_t)4 * CD, 0.0), pq(CNT, 0.0);
    double fX = 1, S2 = -1e300;
    for (int g = 0; g < c.ngrid; g++) {
        const int k = g % CNK, q1 = g / CNK, i1 = q1 % c.n1, q0 = q1 / c.n1, i0 = q0 % CD, t = q0 / CD;
        const int idx[4] = {i0, i1, k / CD, k % CD};
        double e = lnfXs[g] - S2;
        if (e > 10) {
            e = e < 200 ? std::exp(-e) : 0;
            fX = fX * e + 1;
            for (double &v : pp) v *= e;
            for (double &v : pq) v *= e;
            for (int j = 0; j < 4; j++) pp[j * CD + idx[j]] += 1;
            pq[t] += 1;
            S2 = lnfXs[g];
        } else if (e > -200) {
            e = std::exp(e);
            fX += e;
            for (int j = 0; j < 4; j++) pp[j * CD + idx[j]] += e;
            pq[t] += e;
        }
    }
    const double lfX = std::log(fX) + S2;
    if (lnfX_out) {
        lnfX_out[0] = lfX + S1 - (model_d ? 6 : 5) * std::log((double)CD);
        lnfX_out[1] = S1;
        lnfX_out[2] = S2;
    }
    if (grid_out)
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < CD; k++) grid_out[j * CD + k] = (j == 1 && !model_d) ? -1.0 : pp[j * CD + k] / fX;
    if (p0p1_out)
        for (int k = 0; k < CNT; k++) p0p1_out[k] = pq[k] / fX;
    if (post_out) {
        std::vector<double2> wt(c.ngrid);
        for (int g = 0; g < c.ngrid; g++) {
            const double lw = lnfXs[g] - lfX;
            wt[g] = make_double2(std::exp(lw), std::exp(-300 - lw));
        }
        CK(cudaMemcpyAsync(B.wt, wt.data(), sizeof(double2) * c.ngrid, cudaMemcpyHostToDevice, st));
        clade_post_kernel<<<(npatt + 7) / 8, 256, 0, st>>>(c, B.F, B.ptri, B.wt, npatt, B.post);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(post_out, B.post, sizeof(double) * 3 * npatt, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaEventRecord(h->ev1, st));
    CK(cudaStreamSynchronize(st));
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        stats->ms_device = ms;
        stats->ms_host = now_ms() - t0;
        stats->kernels = post_out ? 3 : 2;
        stats->nscale = h->nscale;
        stats->h2d_bytes = sizeof(double) * ((double)c.nsets * npatt + 3 * CNT + (post_out ? 2.0 * c.ngrid : 0));
        stats->d2h_bytes = sizeof(double) * ((double)npatt + c.ngrid + (post_out ? 3.0 * npatt : 0));
    }
    return GB_OK;
}

// The whole clade BEB from the branch lengths, kappa and the branch types'
// Qfactors at the MLE (as codeml's lfunNSsites_ACD reads them): the log f
// tables from gb_beb_tables on the clade grids (get_grid_para_like_ACD
// codeml.c:6457-6473) -- clade C: sets 0..10 from w0 in (0, 1) and w = 1,
// 11..110 from the (0, 3) grids of w2 and w3; clade D: w0 in (0, 0.5), w1 in
// (0.5, 1.5), then the (0, 3) pairs -- followed by gb_beb_clade.
int gb_beb_clade_bl(gb_handle *h, int model_d, const double *blength, double kappa, const double qfactor[2],
                    double *post, double *grid, double *p0p1, double *lnfX, gb_stats *stats) {
    using namespace gb;
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!blength || !qfactor) return fail(GB_ERR_ARG, "null argument");
    const size_t np = (size_t)h->npatt;
    const int nsets = model_d ? 120 : 111;
    std::vector<double> t((size_t)121 * np), L((size_t)nsets * np);
    double g[GB_BEB_GRID], ga[GB_BEB_GRID], gb3[GB_BEB_GRID];
    for (int k = 0; k < GB_BEB_GRID; k++) {
        g[k] = (k + 0.5) / GB_BEB_GRID;
        gb3[k] = 3.0 * g[k];
    }
    // rows [r0, r1) of one gb_beb_tables call into L from row dst
    auto tables = [&](const double *w0, const double *w2, int r0, int r1, int dst) -> int {
        const int rc = gb_beb_tables(h, blength, kappa, qfactor, w0, w2, t.data(), nullptr);
        if (rc) return rc;
        std::copy(t.begin() + (size_t)r0 * np, t.begin() + (size_t)r1 * np, L.begin() + (size_t)dst * np);
        return 0;
    };
    int rc;
    if (!model_d) {
        if ((rc = tables(g, gb3, 0, 11, 0)) || (rc = tables(gb3, gb3, 11, 111, 11))) return rc;
    } else {
        for (int k = 0; k < GB_BEB_GRID; k++) ga[k] = 0.5 * g[k];
        if ((rc = tables(ga, gb3, 0, 10, 0))) return rc;
        for (int k = 0; k < GB_BEB_GRID; k++) ga[k] = 0.5 + g[k];
        if ((rc = tables(ga, gb3, 0, 10, 10)) || (rc = tables(gb3, gb3, 11, 111, 20))) return rc;
    }
    return gb_beb_clade(h, model_d, L.data(), post, grid, p0p1, lnfX, stats);
}
