// Bayes empirical Bayes (BEB) site analysis of branch-site model A on the
// device: the work of codeml's lfunNSsites_ACD (codeml.c:6617-6826).
//
// 1. f(x_h | w) for 121 omega sets (get_grid_para_like_ACD codeml.c:6419-6530).
//    A set gives the background and the foreground branches their own omega;
//    kappa, the branch lengths and the two branch Qfactors stay at the MLE
//    (GetPMatBranch's BEB branch, treesub.c:7289-7301, applies
//    Qfactor_NS_branch to t with the unscaled Q of the set's omega).  The
//    handle's FP64 forward already computes four such sets per launch: its
//    site classes 0 and 1 are full trees with one omega everywhere, and
//    classes 2a and 2b re-prune only the foreground branch's path to the root
//    from class 0 / class 1 subtrees.  So with the three eigen slots set to
//    (w0_i, 1, w2_j) one launch yields sets i, 10, 11 + 10 i + j and 111 + j,
//    and each later (i, j) runs only the items of the classes whose set is
//    new: one forward of all four classes, 9 full class-0 trees (with their
//    class-2a paths), 9 paths of classes 2a + 2b and 81 class-2a paths, each
//    a replayed CUDA graph; the eigen solutions of the 21 omega values are
//    uploaded once and copied into the parameter block on the device between
//    launches.
// 2. Per pattern, the 121 log values are rescaled by their maximum (the S1
//    term), the 10^4-point grid integral log f(X) (get_pclassM_iw_ACD
//    6532-6615, then 6700-6756) and the site-class posteriors (6758-6775).
//    The marginal over the grid with codeml's running scale S2 is a short
//    sequential loop over 10^4 numbers on the host; the two 10^4 x npatt
//    reductions are device kernels.
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

#include "gbcodeml.h"
#include "handle.h"
#include "internal.h"
#include "model.h"

namespace gb {
namespace {

constexpr int BD = GB_BEB_GRID;                 // grid points per dimension
constexpr int BNW = GB_BEB_OMEGA_SETS;          // omega sets
constexpr int BNE = 2 * BD + 1;                 // distinct omega values: w0 grid, 1, w2 grid
constexpr int BNT = BD * BD;                    // (p0, p1) triangles
constexpr int BNG = BNT * BD * BD;              // grid points (triangle, w0, w2)
constexpr int EIG = 2 * NC * NC + NC;           // U, V, Root of one omega
static_assert(BNW == BD + 1 + BD * BD + BD, "omega set count");

// log table (in place, when the forward wrote linear f), per-pattern maximum
// and the rescaled table exp(log f - max)
__global__ void __launch_bounds__(256) beb_rescale_kernel(double *__restrict__ lnfw, double *__restrict__ F,
                                                          double *__restrict__ mrow, int npatt, int npad,
                                                          int linear) {
    const int h = blockIdx.x * blockDim.x + threadIdx.x;
    if (h >= npatt) return;
    double m = 0.0;
    for (int k = 0; k < BNW; k++) {
        double v = lnfw[(size_t)k * npad + h];
        if (linear) {
            v = log(v);
            lnfw[(size_t)k * npad + h] = v;
        }
        if (k == 0 || v > m) m = v;
    }
    for (int k = 0; k < BNW; k++) F[(size_t)k * npad + h] = exp(lnfw[(size_t)k * npad + h] - m);
    mrow[h] = m;
}

// the omega sets the four classes read at grid point g = ((t * 10) + i) * 10 + j
// (t: (p0, p1) triangle, i: w0 index, j: w2 index)
__device__ __forceinline__ void beb_sets(int g, int &t, int &s0, int &s2a, int &s2b) {
    t = g / (BD * BD);
    const int q = g - t * BD * BD;
    const int i = q / BD;
    s0 = i;
    s2a = BD + 1 + q;
    s2b = BD + 1 + BD * BD + (q - i * BD);
}

// lnfXs[g] = sum_h fpatt_h log sum_k p_k(g) F[set_k(g)][h]; one block per grid point
__global__ void __launch_bounds__(256) beb_grid_kernel(const double *__restrict__ F,
                                                       const double *__restrict__ fpatt,
                                                       const double *__restrict__ pcl, int npatt, int npad,
                                                       double *__restrict__ lnfXs) {
    __shared__ double red[8];
    const int g = blockIdx.x;
    int t, s0, s2a, s2b;
    beb_sets(g, t, s0, s2a, s2b);
    const double p0 = pcl[t * 4 + 0], p1 = pcl[t * 4 + 1], p2 = pcl[t * 4 + 2], p3 = pcl[t * 4 + 3];
    const double *r0 = F + (size_t)s0 * npad, *r1 = F + (size_t)BD * npad;
    const double *r2 = F + (size_t)s2a * npad, *r3 = F + (size_t)s2b * npad;
    double s = 0.0;
    for (int h = threadIdx.x; h < npatt; h += blockDim.x) {
        double fh = p0 * r0[h];
        fh += p1 * r1[h];
        fh += p2 * r2[h];
        fh += p3 * r3[h];
        if (fh < 1e-300) continue;   // codeml skips such a pattern ("strange: f[h] very small")
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

// post[k][h] = sum_g [ratio > thr_g] ratio * w_g, ratio = p_k F_k / sum_k p_k F_k and
// w_g = exp(lnfXs[g] - log f(X)): codeml's sum of exp(log(ratio) + lnfXs[g] - log f(X))
// over the terms above exp(-300).  One warp per pattern, lanes over the grid.
__global__ void __launch_bounds__(256) beb_post_kernel(const double *__restrict__ F,
                                                       const double *__restrict__ pcl,
                                                       const double2 *__restrict__ wt, int npatt, int npad,
                                                       double *__restrict__ post) {
    __shared__ double fs[8][BNW + 7];
    __shared__ double ps[BNT * 4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < BNT * 4; i += blockDim.x) ps[i] = pcl[i];
    const int h = blockIdx.x * 8 + warp;
    if (h < npatt)
        for (int k = lane; k < BNW; k += 32) fs[warp][k] = F[(size_t)k * npad + h];
    __syncthreads();
    if (h >= npatt) return;
    const double *f = fs[warp];
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    for (int g = lane; g < BNG; g += 32) {
        int t, s0, s2a, s2b;
        beb_sets(g, t, s0, s2a, s2b);
        const double2 w = wt[g];
        const double f0 = ps[t * 4 + 0] * f[s0], f1 = ps[t * 4 + 1] * f[BD];
        const double f2 = ps[t * 4 + 2] * f[s2a], f3 = ps[t * 4 + 3] * f[s2b];
        const double inv = 1.0 / (((f0 + f1) + f2) + f3);
        double r = f0 * inv;
        if (r > w.y) a0 += r * w.x;
        r = f1 * inv;
        if (r > w.y) a1 += r * w.x;
        r = f2 * inv;
        if (r > w.y) a2 += r * w.x;
        r = f3 * inv;
        if (r > w.y) a3 += r * w.x;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, o);
        a1 += __shfl_down_sync(0xffffffffu, a1, o);
        a2 += __shfl_down_sync(0xffffffffu, a2, o);
        a3 += __shfl_down_sync(0xffffffffu, a3, o);
    }
    if (lane == 0) {
        post[h] = a0;
        post[(size_t)npad + h] = a1;
        post[(size_t)2 * npad + h] = a2;
        post[(size_t)3 * npad + h] = a3;
    }
}

// posterior mean and second moment of the site's w: sum_g w_g sum_k ratio_k w_k(g)
// (and w_k(g)^2), w_k the class's w at grid point g -- w0_i, 1, and w2_j for
// both 2a and 2b (the foreground w; on an all-foreground tree the w of M2a's
// class 2).  codeml's lfunNSsites_M2M8 (codeml.c:6331-6374) drops terms with
// ratio w_k below 1e-300.  Same layout as beb_post_kernel; wv: the 21 w values.
__global__ void __launch_bounds__(256) beb_omega_kernel(const double *__restrict__ F,
                                                        const double *__restrict__ pcl,
                                                        const double2 *__restrict__ wt,
                                                        const double *__restrict__ wv, int npatt, int npad,
                                                        double *__restrict__ mom) {
    __shared__ double fs[8][BNW + 7];
    __shared__ double ps[BNT * 4];
    __shared__ double ws[BNE];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < BNT * 4; i += blockDim.x) ps[i] = pcl[i];
    if (threadIdx.x < BNE) ws[threadIdx.x] = wv[threadIdx.x];
    const int h = blockIdx.x * 8 + warp;
    if (h < npatt)
        for (int k = lane; k < BNW; k += 32) fs[warp][k] = F[(size_t)k * npad + h];
    __syncthreads();
    if (h >= npatt) return;
    const double *f = fs[warp];
    double m1 = 0.0, m2 = 0.0;
    for (int g = lane; g < BNG; g += 32) {
        int t, s0, s2a, s2b;
        beb_sets(g, t, s0, s2a, s2b);
        const double w = wt[g].x;
        const double f0 = ps[t * 4 + 0] * f[s0], f1 = ps[t * 4 + 1] * f[BD];
        const double f2 = ps[t * 4 + 2] * f[s2a], f3 = ps[t * 4 + 3] * f[s2b];
        const double inv = 1.0 / (((f0 + f1) + f2) + f3);
        const double om[4] = {ws[s0], 1.0, ws[s2b - BD * BD], ws[s2b - BD * BD]};
        const double r[4] = {f0 * inv, f1 * inv, f2 * inv, f3 * inv};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const double a = r[k] * om[k];
            if (a >= 1e-300) {
                m1 = fma(a, w, m1);
                m2 = fma(a * om[k], w, m2);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        m1 += __shfl_down_sync(0xffffffffu, m1, o);
        m2 += __shfl_down_sync(0xffffffffu, m2, o);
    }
    if (lane == 0) {
        mom[h] = m1;
        mom[(size_t)npad + h] = m2;
    }
}

// device scratch of one gb_beb call, freed on every exit
struct BebBuffers {
    double *eig = nullptr, *lnfw = nullptr, *F = nullptr, *mrow = nullptr, *pcl = nullptr;
    double *lnfXs = nullptr, *post = nullptr, *wv = nullptr, *mom = nullptr;
    double2 *wt = nullptr;
    ~BebBuffers() {
        void *p[] = {eig, lnfw, F, mrow, pcl, lnfXs, post, wt, wv, mom};
        for (void *q : p)
            if (q) cudaFree(q);
    }
};

// CUDA graph of the forward restricted to the items of the classes in mask
// (bit c: class c): P(t) of every (branch, omega) pair, then those items level
// by level.  Items read their children's slots of the class they depend on
// (classes 2a / 2b read clean subtrees from classes 0 / 1), so a mask runs
// correctly when the classes it leaves out are already in place.
int ensure_cls_graph(gb_handle *h, int mask) {
    if (h->graph_cls[mask]) return 0;
    std::vector<Item> sel;
    std::vector<int> &off = h->cls_off[mask];
    off.assign(h->level_off.size(), 0);
    for (size_t L = 0; L + 1 < h->level_off.size(); L++) {
        off[L] = (int)sel.size();
        for (int i = h->level_off[L]; i < h->level_off[L + 1]; i++)
            if ((mask >> h->items[i].cls) & 1) sel.push_back(h->items[i]);
    }
    off.back() = (int)sel.size();
    int rc = dalloc(&h->d_items_cls[mask], sel.size());
    if (rc) return rc;
    CK(cudaMemcpy(h->d_items_cls[mask], sel.data(), sizeof(Item) * sel.size(), cudaMemcpyHostToDevice));
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int nk = 1;
    launch_pmat_fp64(h->d_pairs, (int)h->pairs.size(), h->d_label, h->d_tnode, h->d_prm, h->d_Pt, h->stream,
                     h->d_pi);
    for (size_t L = 0; L + 1 < off.size(); L++) {
        const int n = off[L + 1] - off[L];
        if (n == 0) continue;
        launch_prune_fp64(h->d_items_cls[mask] + off[L], n, h->ntile, h->npad, h->d_z, h->d_Pt, h->d_conP,
                          nullptr, h->d_scaleF, h->d_scale_list, h->nscale, h->d_pi, h->d_fbar, h->d_ssum,
                          h->d_fhK, h->stream, h->d_amb);
        nk++;
    }
    CK(cudaStreamEndCapture(h->stream, &g));
    cudaError_t e = cudaGraphInstantiate(&h->graph_cls[mask], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(GB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    h->graph_cls_kernels[mask] = nk;
    return 0;
}

// class proportions at the centroid of (p0, p1) triangle t of the ternary plot
// (GetIndexTernary tools.c:4441-4461); 2a and 2b split p2 in the ratio p0 : p1
void triangle_classes(int t, double p[4]) {
    const int ix = (int)std::sqrt((double)t), iy = t - ix * ix;
    const double a = (1 + (iy / 2) * 3 + (iy % 2)) / (3. * BD);
    const double b = (1 + (BD - 1 - ix) * 3 + (iy % 2)) / (3. * BD);
    const double c = 1 - a - b;
    p[0] = a;
    p[1] = b;
    p[2] = c * a / (1 - c);
    p[3] = c * b / (1 - c);
}

}  // namespace
}  // namespace gb

using namespace gb;

int gb_beb(gb_handle *h, const gb_params *prm, double *lnfw_out, double *post_out, double *grid_out,
           double *p0p1_out, double *lnfX_out, gb_stats *stats) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!prm || !prm->blength) return fail(GB_ERR_ARG, "null argument");
    // the branch Qfactors of model A at prm (SetParametersNSsites codeml.c:2490-2512)
    std::vector<Derived> Dv(1);
    ModelParams m{prm->kappa, prm->omega0, prm->omega2, prm->p0, prm->p1};
    int rc = derive_scalars(h->pi.data(), m, &Dv[0]);
    if (rc) return fail(rc, "model parameters out of range");
    return gb_beb_qf(h, prm->blength, prm->kappa, Dv[0].qf, lnfw_out, post_out, grid_out, p0p1_out, lnfX_out,
                     nullptr, nullptr, stats);
}

namespace gb {
namespace {
// the BEB pipeline; wg0 / wg2 (both or neither): the omega grids of eigen
// slots 0 and 2 in place of w0 in (0, 1) and w2 in (1, 11); tables_only:
// stop after the 121 log f tables (no grid integration)
int beb_run(gb_handle *h, const double *blength, double kappa, const double qfactor[2], const double *wg0,
            const double *wg2, bool tables_only, double *lnfw_out, double *post_out, double *grid_out,
            double *p0p1_out, double *lnfX_out, double *wmean_out, double *wsd_out, gb_stats *stats) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!blength || !qfactor) return fail(GB_ERR_ARG, "null argument");
    if (h->precision != GB_PREC_FP64) return fail(GB_ERR_STATE, "gb_beb needs a GB_PREC_FP64 handle");
    if (!(kappa > 0) || !(qfactor[0] > 0) || !(qfactor[1] > 0)) return fail(GB_ERR_PARAM, "kappa or Qfactor");
    const double t0 = now_ms();
    int rc = 0;
    // eigen solutions of the 21 omega values (unscaled Q; the Qfactors scale t)
    std::vector<Derived> Dv(1);
    Derived &D = Dv[0];
    D.qf[0] = qfactor[0];
    D.qf[1] = qfactor[1];
    D.freqK[0] = D.freqK[1] = D.freqK[2] = D.freqK[3] = 0.25;   // the forward's mixture is not used
    double wv[BNE];
    for (int i = 0; i < BD; i++) {
        wv[i] = wg0 ? wg0[i] : (i + 0.5) / BD;                          // w0 in (0, 1)
        wv[BD + 1 + i] = wg2 ? wg2[i] : 1 + (i + 0.5) * (11 - 1) / BD;  // w2 in (1, 11)
        if (!(wv[i] >= 0) || !(wv[BD + 1 + i] >= 0)) return fail(GB_ERR_PARAM, "omega grid");
    }
    wv[BD] = 1;
    std::vector<double> eig((size_t)BNE * EIG);
    for (int e = 0; e < BNE; e++) {
        std::vector<double> Q(NC * NC);
        build_q(h->pi.data(), kappa, wv[e], Q.data(), nullptr, nullptr);
        double *E = &eig[(size_t)e * EIG];
        if (eigen_qrev(Q.data(), h->pi.data(), E, E + NC * NC, E + 2 * NC * NC))
            return fail(GB_ERR_PARAM, "eigen solution failed");
    }
    // the parameter block starts as (w0_0, 1, w2_0) with the Qfactors of prm
    for (int s = 0; s < 3; s++) {
        const int e = s == 0 ? 0 : (s == 1 ? BD : BD + 1);
        std::memcpy(D.U[s], &eig[(size_t)e * EIG], sizeof(double) * NC * NC);
        std::memcpy(D.V[s], &eig[(size_t)e * EIG + NC * NC], sizeof(double) * NC * NC);
        std::memcpy(D.Root[s], &eig[(size_t)e * EIG + 2 * NC * NC], sizeof(double) * NC);
    }
    D.sym = 1;
    if ((rc = stage_params(h, &D, blength))) return rc;
    if ((rc = fp64_prepare(h, false))) return rc;
    // class masks: 2a + 2b on the path; 0 + 2a for a new w0 (class 1 and
    // class 2b do not depend on w0); 2a alone for a new w2 under the same w0
    constexpr int M_PATH = 0xC, M_W0 = 0x5, M_2A = 0x4;
    for (int mask : {M_PATH, M_W0, M_2A})
        if ((rc = ensure_cls_graph(h, mask))) return rc;
    const size_t npad = h->npad;
    const int npatt = h->npatt;
    BebBuffers B;
    if ((rc = dalloc(&B.eig, eig.size())) || (rc = dalloc(&B.lnfw, (size_t)BNW * npad)) ||
        (rc = dalloc(&B.F, (size_t)BNW * npad)) || (rc = dalloc(&B.mrow, npad)) ||
        (rc = dalloc(&B.pcl, BNT * 4)) || (rc = dalloc(&B.lnfXs, BNG)) || (rc = dalloc(&B.post, 4 * npad)) ||
        (rc = dalloc(&B.wt, BNG)) || (rc = dalloc(&B.wv, BNE)) || (rc = dalloc(&B.mom, 2 * npad)))
        return rc;
    std::vector<double> pcl(BNT * 4);
    for (int t = 0; t < BNT; t++) triangle_classes(t, &pcl[t * 4]);
    cudaStream_t st = h->stream;
    CK(cudaEventRecord(h->ev0, st));
    CK(cudaMemcpyAsync(B.eig, eig.data(), sizeof(double) * eig.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(B.pcl, pcl.data(), sizeof(double) * pcl.size(), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(h->d_prm, h->h_prm, sizeof(DevParams), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(h->d_tnode, h->h_tnode, sizeof(double) * h->nnode, cudaMemcpyHostToDevice, st));
    // eigen slot s of the device parameter block <- omega value e
    char *prm_base = reinterpret_cast<char *>(h->d_prm);
    auto set_slot = [&](int s, int e) -> int {
        const double *E = B.eig + (size_t)e * EIG;
        const size_t mat = sizeof(double) * NC * NC, vec = sizeof(double) * NC;
        CK(cudaMemcpyAsync(prm_base + offsetof(DevParams, U) + s * mat, E, mat, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(prm_base + offsetof(DevParams, V) + s * mat, E + NC * NC, mat,
                           cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(prm_base + offsetof(DevParams, Root) + s * vec, E + 2 * NC * NC, vec,
                           cudaMemcpyDeviceToDevice, st));
        return 0;
    };
    auto keep = [&](int cls, int set) -> int {
        CK(cudaMemcpyAsync(B.lnfw + (size_t)set * npad, h->d_fhK + (size_t)cls * npad, sizeof(double) * npad,
                           cudaMemcpyDeviceToDevice, st));
        return 0;
    };
    // (w0_0, 1, w2_0): every class; then per (i, j) only the classes whose
    // omega set is new: sets i (class 0), 10 (class 1, once), 11 + 10 i + j
    // (class 2a) and 111 + j (class 2b, under w0_0 only)
    int kernels = 0;
    for (int i = 0; i < BD; i++) {
        if ((rc = set_slot(0, i))) return rc;
        for (int j = 0; j < BD; j++) {
            if ((rc = set_slot(2, BD + 1 + j))) return rc;
            const int mask = j == 0 ? (i == 0 ? 0xF : M_W0) : (i == 0 ? M_PATH : M_2A);
            if (mask == 0xF) {
                CK(cudaGraphLaunch(h->graph[0], st));
                kernels += h->graph_kernels;
            } else {
                CK(cudaGraphLaunch(h->graph_cls[mask], st));
                kernels += h->graph_cls_kernels[mask];
            }
            if (j == 0 && (rc = keep(0, i))) return rc;
            if (i == 0 && j == 0 && (rc = keep(1, BD))) return rc;
            if ((rc = keep(2, BD + 1 + i * BD + j))) return rc;
            if (i == 0 && (rc = keep(3, BD + 1 + BD * BD + j))) return rc;
        }
    }
    beb_rescale_kernel<<<(npatt + 255) / 256, 256, 0, st>>>(B.lnfw, B.F, B.mrow, npatt, (int)npad,
                                                            h->nscale == 0);
    if (tables_only) {
        kernels++;
        CK(cudaGetLastError());
        if (lnfw_out)
            CK(cudaMemcpy2DAsync(lnfw_out, sizeof(double) * npatt, B.lnfw, sizeof(double) * npad,
                                 sizeof(double) * npatt, BNW, cudaMemcpyDeviceToHost, st));
        CK(cudaEventRecord(h->ev1, st));
        CK(cudaStreamSynchronize(st));
        CK(cudaGetLastError());
        if (stats) {
            float ms = 0;
            cudaEventElapsedTime(&ms, h->ev0, h->ev1);
            stats->ms_device = ms;
            stats->ms_host = now_ms() - t0;
            stats->kernels = kernels;
            stats->nscale = h->nscale;
            stats->h2d_bytes = sizeof(double) * (eig.size() + pcl.size() + h->nnode) + sizeof(DevParams);
            stats->d2h_bytes = lnfw_out ? sizeof(double) * (size_t)BNW * npatt : 0;
        }
        return GB_OK;
    }
    beb_grid_kernel<<<BNG, 256, 0, st>>>(B.F, h->d_fpatt, B.pcl, npatt, (int)npad, B.lnfXs);
    kernels += 2;
    CK(cudaGetLastError());
    std::vector<double> mrow(npatt), lnfXs(BNG);
    CK(cudaMemcpyAsync(mrow.data(), B.mrow, sizeof(double) * npatt, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(lnfXs.data(), B.lnfXs, sizeof(double) * BNG, cudaMemcpyDeviceToHost, st));
    if (lnfw_out)
        CK(cudaMemcpy2DAsync(lnfw_out, sizeof(double) * npatt, B.lnfw, sizeof(double) * npad,
                             sizeof(double) * npatt, BNW, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    // S1, then the marginal over the grid with codeml's running scale S2
    // (lfunNSsites_ACD codeml.c:6700-6747): a new largest term rescales the sum
    double S1 = 0;
    for (int hh = 0; hh < npatt; hh++) S1 += mrow[hh] * h->fpatt[hh];
    double pp[4][BD], pq[BNT];
    std::memset(pp, 0, sizeof pp);
    std::memset(pq, 0, sizeof pq);
    double fX = 1, S2 = -1e300;
    for (int g = 0; g < BNG; g++) {
        int ip[4];
        for (int j = 3, it = g; j >= 0; j--) { ip[j] = it % BD; it /= BD; }
        double t = lnfXs[g] - S2;
        if (t > 10) {
            t = t < 200 ? std::exp(-t) : 0;
            fX = fX * t + 1;
            for (int j = 0; j < 4; j++)
                for (int k = 0; k < BD; k++) pp[j][k] *= t;
            for (int k = 0; k < BNT; k++) pq[k] *= t;
            for (int j = 0; j < 4; j++) pp[j][ip[j]] += 1;
            pq[ip[0] * BD + ip[1]] += 1;
            S2 = lnfXs[g];
        } else if (t > -200) {
            t = std::exp(t);
            fX += t;
            for (int j = 0; j < 4; j++) pp[j][ip[j]] += t;
            pq[ip[0] * BD + ip[1]] += t;
        }
    }
    const double lfX = std::log(fX) + S2;
    if (lnfX_out) {
        lnfX_out[0] = lfX + S1 - 4 * std::log((double)BD);
        lnfX_out[1] = S1;
        lnfX_out[2] = S2;
    }
    if (grid_out)
        for (int j = 0; j < 4; j++)
            for (int k = 0; k < BD; k++) grid_out[j * BD + k] = j < 2 ? -1.0 : pp[j][k] / fX;
    if (p0p1_out)
        for (int k = 0; k < BNT; k++) p0p1_out[k] = pq[k] / fX;
    const bool want_w = wmean_out || wsd_out;
    std::vector<double2> wt(BNG);
    if (post_out || want_w) {
        for (int g = 0; g < BNG; g++) {
            const double lw = lnfXs[g] - lfX;
            wt[g] = make_double2(std::exp(lw), std::exp(-300 - lw));
        }
        CK(cudaMemcpyAsync(B.wt, wt.data(), sizeof(double2) * BNG, cudaMemcpyHostToDevice, st));
    }
    std::vector<double> mom;
    if (want_w) {
        CK(cudaMemcpyAsync(B.wv, wv, sizeof(double) * BNE, cudaMemcpyHostToDevice, st));
        beb_omega_kernel<<<(npatt + 7) / 8, 256, 0, st>>>(B.F, B.pcl, B.wt, B.wv, npatt, (int)npad, B.mom);
        kernels++;
        CK(cudaGetLastError());
        mom.resize((size_t)2 * npatt);
        CK(cudaMemcpy2DAsync(mom.data(), sizeof(double) * npatt, B.mom, sizeof(double) * npad,
                             sizeof(double) * npatt, 2, cudaMemcpyDeviceToHost, st));
    }
    if (post_out) {
        beb_post_kernel<<<(npatt + 7) / 8, 256, 0, st>>>(B.F, B.pcl, B.wt, npatt, (int)npad, B.post);
        kernels++;
        CK(cudaGetLastError());
        CK(cudaMemcpy2DAsync(post_out, sizeof(double) * npatt, B.post, sizeof(double) * npad,
                             sizeof(double) * npatt, 4, cudaMemcpyDeviceToHost, st));
    }
    CK(cudaEventRecord(h->ev1, st));
    CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    // mean and standard deviation of w (codeml.c:6370-6374)
    for (int hh = 0; want_w && hh < npatt; hh++) {
        const double m1 = mom[hh], m2 = mom[(size_t)npatt + hh] - m1 * m1;
        if (wmean_out) wmean_out[hh] = m1;
        if (wsd_out) wsd_out[hh] = m2 > 0 ? std::sqrt(m2) : 0.0;
    }
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        stats->ms_device = ms;
        stats->ms_host = now_ms() - t0;
        stats->kernels = kernels;
        stats->nscale = h->nscale;
        stats->h2d_bytes = sizeof(double) * (eig.size() + pcl.size() + h->nnode) + sizeof(DevParams) +
                           (post_out || want_w ? sizeof(double2) * BNG : 0);
        stats->d2h_bytes = sizeof(double) * (npatt + BNG + (lnfw_out ? (size_t)BNW * npatt : 0) +
                                             (post_out ? 4 * npatt : 0));
    }
    return GB_OK;
}
}  // namespace
}  // namespace gb

int gb_beb_qf(gb_handle *h, const double *blength, double kappa, const double qfactor[2], double *lnfw_out,
              double *post_out, double *grid_out, double *p0p1_out, double *lnfX_out, double *wmean_out,
              double *wsd_out, gb_stats *stats) {
    return beb_run(h, blength, kappa, qfactor, nullptr, nullptr, false, lnfw_out, post_out, grid_out, p0p1_out,
                   lnfX_out, wmean_out, wsd_out, stats);
}

int gb_beb_tables(gb_handle *h, const double *blength, double kappa, const double qfactor[2],
                  const double w_slot0[GB_BEB_GRID], const double w_slot2[GB_BEB_GRID], double *lnfw,
                  gb_stats *stats) {
    if (!w_slot0 || !w_slot2 || !lnfw) return fail(GB_ERR_ARG, "null argument");
    return beb_run(h, blength, kappa, qfactor, w_slot0, w_slot2, true, lnfw, nullptr, nullptr, nullptr, nullptr,
                   nullptr, nullptr, stats);
}
