// Standard errors and Hessians of model A on the device.
//
// gb_se_opg: what codeml computes with getSE = 1 (codeml.c:754-783): the
// Hessian approximation of HessianSKT2004 (treesub.c:6979-7048), minus the
// fpatt-weighted sum over patterns of the outer products of the per-pattern
// scores d log f_h / dx, each score a central difference with step
// 2 Small_Diff (|x_i| + 1); then SE_i = sqrt([(-H)^-1]_ii).  codeml runs the
// 2 np likelihood evaluations one after the other on one core and keeps
// np x npatt scores in host memory.  Here the 2 np FP64 evaluations are
// replays of the handle's forward graph on one stream, fed from parameter
// blocks and branch-length vectors uploaded once (device-to-device copies
// between replays, no host round trip), each leaving its per-pattern log f in
// a device table; one kernel forms the scores and the np x np product.  Only
// the inverse is on the host.
//
// gb_hessian_x: the Hessian itself, by central differences of the analytic
// gradient (gb_dfun_x), 2 np gradient evaluations instead of the 2 np^2
// likelihood evaluations of codeml's Hessian (tools.c:5774-5810).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "gbcodeml.h"
#include "handle.h"
#include "internal.h"
#include "model.h"

namespace gb {
namespace {

constexpr int HT = 16;       // H tile edge (16 x 16 threads)
constexpr int HK = 64;       // patterns per shared-memory step

// D[i][h] = (L[n + i][h] - L[i][h]) / (2 eh_i): the central-difference score
__global__ void __launch_bounds__(256) opg_scores_kernel(const double *__restrict__ L,
                                                         const double *__restrict__ eh, int n, int npatt,
                                                         int npad, double *__restrict__ D) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = blockIdx.y;
    if (h >= npatt) return;
    D[(size_t)i * npad + h] = (L[(size_t)(n + i) * npad + h] - L[(size_t)i * npad + h]) / (eh[i] * 2);
}

// H[i][j] = -sum_h fpatt_h (D_i(h) D_j(h)); the product D_i D_j is formed
// first, so H[i][j] and H[j][i] are the same sum and H is exactly symmetric
__global__ void __launch_bounds__(HT * HT) opg_product_kernel(const double *__restrict__ D,
                                                              const double *__restrict__ fpatt, int n,
                                                              int npatt, int npad, double *__restrict__ H) {
    __shared__ double A[HT][HK + 1], B[HT][HK + 1], W[HK];
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * HT + tx;
    const int i0 = blockIdx.y * HT, j0 = blockIdx.x * HT;
    double acc = 0.0;
    for (int h0 = 0; h0 < npatt; h0 += HK) {
        for (int e = tid; e < HT * HK; e += HT * HT) {
            const int r = e / HK, c = e % HK, h = h0 + c;
            const bool hin = h < npatt;
            A[r][c] = (hin && i0 + r < n) ? D[(size_t)(i0 + r) * npad + h] : 0.0;
            B[r][c] = (hin && j0 + r < n) ? D[(size_t)(j0 + r) * npad + h] : 0.0;
            if (r == 0) W[c] = hin ? fpatt[h] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int c = 0; c < HK; c++) acc = fma(W[c], A[ty][c] * B[tx][c], acc);
        __syncthreads();
    }
    const int i = i0 + ty, j = j0 + tx;
    if (i < n && j < n) H[(size_t)i * n + j] = -acc;
}

// inverse of an n x n matrix by Gauss-Jordan elimination with partial
// pivoting (the method of codeml's matinv); false if singular
bool invert(std::vector<double> &a, int n) {
    std::vector<int> piv(n);
    for (int k = 0; k < n; k++) {
        int p = k;
        for (int r = k + 1; r < n; r++)
            if (std::fabs(a[(size_t)r * n + k]) > std::fabs(a[(size_t)p * n + k])) p = r;
        if (a[(size_t)p * n + k] == 0.0) return false;
        piv[k] = p;
        if (p != k)
            for (int c = 0; c < n; c++) std::swap(a[(size_t)k * n + c], a[(size_t)p * n + c]);
        const double d = 1.0 / a[(size_t)k * n + k];
        a[(size_t)k * n + k] = 1.0;
        for (int c = 0; c < n; c++) a[(size_t)k * n + c] *= d;
        for (int r = 0; r < n; r++) {
            if (r == k) continue;
            const double f = a[(size_t)r * n + k];
            if (f == 0.0) continue;
            a[(size_t)r * n + k] = 0.0;
            for (int c = 0; c < n; c++) a[(size_t)r * n + c] -= f * a[(size_t)k * n + c];
        }
    }
    for (int k = n - 1; k >= 0; k--)
        if (piv[k] != k)
            for (int r = 0; r < n; r++) std::swap(a[(size_t)r * n + k], a[(size_t)r * n + piv[k]]);
    return true;
}

// SE_i = sqrt(C_ii) of C = M^-1, -1 where C_ii is not positive (codeml.c:780-782)
int standard_errors(const double *M, int n, double *se) {
    std::vector<double> a(M, M + (size_t)n * n);
    if (!invert(a, n)) {
        for (int i = 0; i < n; i++) se[i] = -1.0;
        return fail(GB_ERR_PARAM, "singular Hessian");
    }
    for (int i = 0; i < n; i++) {
        const double v = a[(size_t)i * n + i];
        se[i] = v > 0.0 ? std::sqrt(v) : -1.0;
    }
    return 0;
}

struct SeBuffers {
    DevParams *prm = nullptr;
    double *T = nullptr, *L = nullptr, *D = nullptr, *eh = nullptr, *H = nullptr, *lnL = nullptr;
    ~SeBuffers() {
        void *p[] = {prm, T, L, D, eh, H, lnL};
        for (void *q : p)
            if (q) cudaFree(q);
    }
};

void to_devparams(const Derived &D, DevParams *P) {
    std::memcpy(P->U, D.U, sizeof(D.U));
    std::memcpy(P->V, D.V, sizeof(D.V));
    std::memcpy(P->Root, D.Root, sizeof(D.Root));
    std::memcpy(P->qf, D.qf, sizeof(D.qf));
    std::memcpy(P->freqK, D.freqK, sizeof(D.freqK));
    P->sym = D.sym;
}

}  // namespace
}  // namespace gb

using namespace gb;

int gb_se_opg(gb_handle *h, const int *bnode, const double *x, int n, double small_diff, double *g,
              double *H_out, double *se, gb_stats *stats) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (h->precision != GB_PREC_FP64) return fail(GB_ERR_STATE, "gb_se_opg needs a GB_PREC_FP64 handle");
    const int nb = h->nnode - 1;
    // model A: x ends kappa, p0, p1, w0, w2; model B (n = nb + 6): ..., w0, w1, w2
    if (!bnode || !x || (n != nb + 5 && n != nb + 6) || !(small_diff > 0))
        return fail(GB_ERR_ARG, "gb_se_opg: bad arguments");
    const int nm = n - nb;             // model parameters
    const bool model_b = nm == 6;
    for (int ib = 0; ib < nb; ib++)
        if (bnode[ib] < 0 || bnode[ib] >= h->nnode || bnode[ib] == h->root) return fail(GB_ERR_ARG, "bnode");
    const double t0 = now_ms();
    std::vector<double> eh(n);
    for (int i = 0; i < n; i++) eh[i] = small_diff * 2 * (std::fabs(x[i]) + 1);
    // parameter blocks: [0] at x, [1 + 2 q + bf] with model parameter q moved by -eh (bf 0) / +eh (bf 1)
    std::vector<DevParams> P(1 + 2 * nm);
    std::vector<Derived> Dv(1);
    auto model_at = [&](const double *xv, DevParams *out) -> int {
        ModelParams m{xv[nb], xv[nb + 3], xv[n - 1], xv[nb + 1], xv[nb + 2]};
        if (model_b) {
            m.w1 = xv[nb + 4];
            m.free_w1 = true;
        }
        int rc = derive(h->pi.data(), m, false, &Dv[0]);
        if (rc) return fail(rc, "model parameters out of range");
        to_devparams(Dv[0], out);
        return 0;
    };
    int rc = model_at(x, &P[0]);
    if (rc) return rc;
    std::vector<double> xs(x, x + n);
    for (int q = 0; q < nm; q++)
        for (int bf = 0; bf < 2; bf++) {
            xs[nb + q] = x[nb + q] + (bf ? eh[nb + q] : -eh[nb + q]);
            rc = model_at(xs.data(), &P[1 + 2 * q + bf]);
            xs[nb + q] = x[nb + q];
            if (rc) return rc;
        }
    // branch lengths (node order) of evaluation k = bf * n + i; a length moved
    // below zero acts as zero (P = I, as PMatUVRoot does for t < 1e-100)
    const int ne = 2 * n;
    std::vector<double> T((size_t)ne * h->nnode, 0.0);
    for (int k = 0; k < ne; k++) {
        const int bf = k / n, i = k % n;
        double *t = &T[(size_t)k * h->nnode];
        for (int ib = 0; ib < nb; ib++) t[bnode[ib]] = x[ib];
        if (i < nb) t[bnode[i]] = x[i] + (bf ? eh[i] : -eh[i]);
    }
    // the forward graph reads the handle's parameter block and branch lengths
    for (int ib = 0; ib < nb; ib++)
        if (!(x[ib] >= 0.0) || !std::isfinite(x[ib])) return fail(GB_ERR_PARAM, "negative or non-finite branch length");
    if ((rc = fp64_prepare(h, false))) return rc;
    const size_t npad = h->npad;
    SeBuffers B;
    if ((rc = dalloc(&B.prm, P.size())) || (rc = dalloc(&B.T, T.size())) || (rc = dalloc(&B.L, (size_t)ne * npad)) ||
        (rc = dalloc(&B.D, (size_t)n * npad)) || (rc = dalloc(&B.eh, n)) ||
        (rc = dalloc(&B.H, (size_t)n * n)) || (rc = dalloc(&B.lnL, ne)))
        return rc;
    cudaStream_t st = h->stream;
    CK(cudaEventRecord(h->ev0, st));
    CK(cudaMemcpyAsync(B.prm, P.data(), sizeof(DevParams) * P.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B.T, T.data(), sizeof(double) * T.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B.eh, eh.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    int loaded = -1, kernels = 0;
    for (int k = 0; k < ne; k++) {
        const int bf = k / n, i = k % n;
        const int want = i < nb ? 0 : 1 + 2 * (i - nb) + bf;
        if (want != loaded) {
            CK(cudaMemcpyAsync(h->d_prm, B.prm + want, sizeof(DevParams), cudaMemcpyDeviceToDevice, st));
            loaded = want;
        }
        CK(cudaMemcpyAsync(h->d_tnode, B.T + (size_t)k * h->nnode, sizeof(double) * h->nnode,
                           cudaMemcpyDeviceToDevice, st));
        CK(cudaGraphLaunch(h->graph[0], st));
        kernels += h->graph_kernels;
        CK(cudaMemcpyAsync(B.L + (size_t)k * npad, h->d_lnf, sizeof(double) * npad, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(B.lnL + k, h->d_out, sizeof(double), cudaMemcpyDeviceToDevice, st));
    }
    opg_scores_kernel<<<dim3((h->npatt + 255) / 256, n), 256, 0, st>>>(B.L, B.eh, n, h->npatt, (int)npad, B.D);
    dim3 tiles((n + HT - 1) / HT, (n + HT - 1) / HT);
    opg_product_kernel<<<tiles, dim3(HT, HT), 0, st>>>(B.D, h->d_fpatt, n, h->npatt, (int)npad, B.H);
    kernels += 2;
    CK(cudaGetLastError());
    std::vector<double> H((size_t)n * n), nl(ne);
    CK(cudaMemcpyAsync(H.data(), B.H, sizeof(double) * H.size(), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(nl.data(), B.lnL, sizeof(double) * ne, cudaMemcpyDeviceToHost, st));
    CK(cudaEventRecord(h->ev1, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    // g from the same lnL differences (d_out holds -lnL)
    if (g)
        for (int i = 0; i < n; i++) g[i] = (-nl[n + i] + nl[i]) / (eh[i] * 2);
    if (H_out) std::memcpy(H_out, H.data(), sizeof(double) * H.size());
    rc = 0;
    if (se) {
        for (double &v : H) v = -v;
        rc = standard_errors(H.data(), n, se);
    }
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        stats->ms_device = ms;
        stats->ms_host = now_ms() - t0;
        stats->kernels = kernels;
        stats->nscale = h->nscale;
        stats->h2d_bytes = sizeof(DevParams) * P.size() + sizeof(double) * (T.size() + n);
        stats->d2h_bytes = sizeof(double) * ((size_t)n * n + ne);
    }
    return rc;
}

int gb_hessian_x(gb_handle *h, const int *bnode, int lastround, const double *x, int n, double rel_step,
                 double *H, double *se) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!bnode || !x || !H || (n != h->nnode - 1 + 5 && n != h->nnode - 1 + 6))
        return fail(GB_ERR_ARG, "gb_hessian_x: bad arguments");
    if (!(rel_step > 0)) rel_step = 1e-5;
    std::vector<double> xs(x, x + n), gp(n), gm(n);
    double f = 0;
    for (int i = 0; i < n; i++) {
        const double s = rel_step * (std::fabs(x[i]) + 1);
        xs[i] = x[i] + s;
        int rc = gb_dfun_x(h, bnode, lastround, xs.data(), n, &f, gp.data());
        if (rc) return rc;
        xs[i] = x[i] - s;
        rc = gb_dfun_x(h, bnode, lastround, xs.data(), n, &f, gm.data());
        if (rc) return rc;
        xs[i] = x[i];
        for (int j = 0; j < n; j++) H[(size_t)i * n + j] = (gp[j] - gm[j]) / (2 * s);
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < i; j++) {
            const double v = 0.5 * (H[(size_t)i * n + j] + H[(size_t)j * n + i]);
            H[(size_t)i * n + j] = H[(size_t)j * n + i] = v;
        }
    return se ? standard_errors(H, n, se) : 0;
}

// codeml's getSE = 1 estimator under the clade models C and D: x = branch
// lengths (codeml's branch order), kappa, p0, p1 (untransformed), w0, [w1
// under D], w2, w3.  The 2n evaluations are gb_eval_clade calls (one graph
// each), their per-pattern log f copied back; the scores and the outer
// product on the host (n^2 npatt operations).
int gb_se_opg_clade(gb_handle *h, const int *bnode, int model_d, const double *x, int n, double small_diff,
                    double *g, double *H_out, double *se) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    const int nb = h->nnode - 1;
    if (!bnode || !x || n != nb + (model_d ? 7 : 6) || !(small_diff > 0))
        return fail(GB_ERR_ARG, "gb_se_opg_clade: bad arguments");
    const int np = h->npatt;
    std::vector<double> eh(n), xs(x, x + n), bl(h->nnode, 0.0), lnf(np);
    std::vector<double> D((size_t)n * np), lnL(2 * n);
    for (int i = 0; i < n; i++) eh[i] = small_diff * 2 * (std::fabs(x[i]) + 1);
    for (int i = 0; i < n; i++)
        for (int bf = 0; bf < 2; bf++) {
            xs[i] = x[i] + (bf ? eh[i] : -eh[i]);
            for (int ib = 0; ib < nb; ib++) {
                if (bnode[ib] < 0 || bnode[ib] >= h->nnode || bnode[ib] == h->root) return fail(GB_ERR_ARG, "bnode");
                bl[bnode[ib]] = xs[ib] > 0.0 ? xs[ib] : 0.0;     // a length moved below zero acts as zero
            }
            const double om[4] = {xs[nb + 3], model_d ? xs[nb + 4] : 1.0, xs[n - 2], xs[n - 1]};
            double f = 0;
            const int rc = gb_eval_clade(h, bl.data(), xs[nb], xs[nb + 1], xs[nb + 2], om, &f, nullptr, nullptr,
                                         lnf.data(), nullptr);
            xs[i] = x[i];
            if (rc) return rc;
            lnL[bf * n + i] = -f;
            for (int hh = 0; hh < np; hh++) D[(size_t)i * np + hh] += (bf ? lnf[hh] : -lnf[hh]) / (2 * eh[i]);
        }
    std::vector<double> H((size_t)n * n);
    const double *fp = h->fpatt.data();
    for (int i = 0; i < n; i++)
        for (int j = 0; j <= i; j++) {
            double s = 0;
            for (int hh = 0; hh < np; hh++) s += fp[hh] * D[(size_t)i * np + hh] * D[(size_t)j * np + hh];
            H[(size_t)i * n + j] = H[(size_t)j * n + i] = -s;
        }
    if (g)
        for (int i = 0; i < n; i++) g[i] = (lnL[n + i] - lnL[i]) / (2 * eh[i]);
    if (H_out) std::memcpy(H_out, H.data(), sizeof(double) * H.size());
    if (!se) return GB_OK;
    for (double &v : H) v = -v;
    return standard_errors(H.data(), n, se);
}
