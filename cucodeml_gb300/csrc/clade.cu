// Clade models C and D with two branch types in one evaluation
// (gb_eval_clade_uvr, FP64 handles).
//
// codeml's clade models (model = 3, NSsites = 2 or 3, ncatG = 3;
// SetParametersNSsites codeml.c:2437-2446, Set_UVR_BranchSite codeml.c:2535-2568)
// have three site classes: class 0 with w0 and class 1 with w1 (1 under clade
// C) on every branch, class 2 with w2 on branch type 0 and w3 on branch type
// 1.  Their class 2 differs from classes 0 and 1 on every branch, so unlike
// model A's classes 2a/2b it needs its own conditional likelihoods at every
// internal node.  The schedule here has three classes at every internal node,
// four eigen solutions (w0, w1, w2, w3) and three transition matrices per
// branch (w0, w1, and w2 or w3 by the branch's type), and runs on the FP64
// kernels of the model-A path: P(t) for the pairs of eigen solutions 0..2
// from the handle's parameter block and for those of solution 3 from a second
// block whose slot 0 holds it, the pruning level by level, then codeml's
// mixture with class 3 weighted zero (its fhK row a copy of class 2's, so the
// mixture is that of the three classes).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "handle.h"

namespace gb {

struct CladeState {
    std::vector<Item> items;
    std::vector<int> level_off;
    std::vector<PairDesc> pairs;      // eigen solutions 0..2, then solution 3 (stored as w = 0)
    std::vector<int> scale_list;      // [4][nscale] scale slot per root class and scaled node (row 3 = row 2)
    int n012 = 0, n3 = 0;
    int nslot = 0, nsslot = 0;
    Item *d_items = nullptr;
    PairDesc *d_pairs = nullptr;
    int *d_scale_list = nullptr;
    double *d_Pt = nullptr, *d_conP = nullptr, *d_scaleF = nullptr;
    DevParams *d_prm3 = nullptr, *h_prm3 = nullptr;
    cudaGraphExec_t graph = nullptr;
    int kernels = 0;
};

void clade_free(CladeState *c) {
    if (!c) return;
    if (c->graph) cudaGraphExecDestroy(c->graph);
    void *dev[] = {c->d_items, c->d_pairs, c->d_scale_list, c->d_Pt, c->d_conP, c->d_scaleF, c->d_prm3};
    for (void *p : dev)
        if (p) cudaFree(p);
    if (c->h_prm3) cudaFreeHost(c->h_prm3);
    delete c;
}

namespace {

// the three-class schedule over the handle's tree, heights and scaled nodes
void build_clade_schedule(const gb_handle *h, CladeState *c) {
    const int nn = h->nnode, ns = h->ns;
    std::vector<int> slot_of((size_t)nn * 3, -1), sslot_of((size_t)nn * 3, -1);
    for (int a = ns; a < nn; a++)
        for (int k = 0; k < 3; k++) {
            slot_of[a * 3 + k] = c->nslot++;
            if (h->scale[a]) sslot_of[a * 3 + k] = c->nsslot++;
        }
    // eigen solution of class k on a branch of type lab: w0, w1, then w2 / w3
    auto wof = [](int k, int lab) { return k < 2 ? k : 2 + lab; };
    std::vector<int> pair_of((size_t)nn * 4, -1);
    for (int pass = 0; pass < 2; pass++)
        for (int n = 0; n < nn; n++) {
            if (n == h->root) continue;
            for (int k = 0; k < 3; k++) {
                const int w = wof(k, h->label[n]);
                if ((w == 3) != (pass == 1)) continue;
                pair_of[n * 4 + w] = (int)c->pairs.size();
                c->pairs.push_back(PairDesc{n, w == 3 ? 0 : w});
            }
        }
    c->n3 = 0;
    for (int n = 0; n < nn; n++) c->n3 += (n != h->root && h->label[n] == 1);
    c->n012 = (int)c->pairs.size() - c->n3;
    const int H = h->height[h->root];
    c->level_off.assign(H + 1, 0);
    for (int L = 1; L <= H; L++) {
        c->level_off[L - 1] = (int)c->items.size();
        for (int a = ns; a < nn; a++) {
            if (h->height[a] != L) continue;
            for (int k = 0; k < 3; k++) {
                Item it{};
                it.node = a;
                it.cls = k;
                it.slot = slot_of[a * 3 + k];
                it.nchild = h->nson[a];
                for (int q = 0; q < MAXC; q++) it.child[q] = it.cslot[q] = it.pidx[q] = -1;
                for (int q = 0; q < it.nchild; q++) {
                    const int s = h->sons[a * MAXC + q];
                    it.child[q] = s;
                    it.cslot[q] = s < ns ? -1 : slot_of[s * 3 + k];
                    it.pidx[q] = pair_of[s * 4 + wof(k, h->label[s])];
                }
                it.sslot = h->scale[a] ? sslot_of[a * 3 + k] : -1;
                it.is_root = a == h->root;
                it.eslot = it.slot * MAXC;
                c->items.push_back(it);
            }
        }
    }
    c->level_off[H] = (int)c->items.size();
    c->scale_list.assign((size_t)4 * std::max(h->nscale, 1), 0);
    for (int k = 0; k < 4; k++) {
        int j = 0;
        for (int b = 0; b < nn; b++)
            if (h->scale[b]) c->scale_list[(size_t)k * h->nscale + j++] = sslot_of[b * 3 + (k < 3 ? k : 2)];
    }
}

// device copies of the schedule and the graph of one evaluation
int clade_setup(gb_handle *h, CladeState *c) {
    build_clade_schedule(h, c);
    const std::vector<int> &sl = c->scale_list;
    int rc;
    if ((rc = dalloc(&c->d_items, c->items.size())) || (rc = dalloc(&c->d_pairs, c->pairs.size())) ||
        (rc = dalloc(&c->d_scale_list, sl.size())) || (rc = dalloc(&c->d_Pt, c->pairs.size() * 4096)) ||
        (rc = dalloc(&c->d_conP, (size_t)c->nslot * h->npad * 64)) ||
        (rc = dalloc(&c->d_scaleF, (size_t)std::max(c->nsslot, 1) * h->npad)) || (rc = dalloc(&c->d_prm3, 1)))
        return rc;
    CK(cudaMallocHost((void **)&c->h_prm3, sizeof(DevParams)));
    std::memset(c->h_prm3, 0, sizeof(DevParams));
    CK(cudaMemcpy(c->d_items, c->items.data(), sizeof(Item) * c->items.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_pairs, c->pairs.data(), sizeof(PairDesc) * c->pairs.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_scale_list, sl.data(), sizeof(int) * sl.size(), cudaMemcpyHostToDevice));
    CK(cudaMemset(c->d_scaleF, 0, sizeof(double) * std::max(c->nsslot, 1) * h->npad));
    // one graph: P(t) of both parameter blocks, the pruning level by level,
    // class 3's fhK row from class 2's, the mixture
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int nk = 0;
    launch_pmat_fp64(c->d_pairs, c->n012, h->d_label, h->d_tnode, h->d_prm, c->d_Pt, h->stream);
    nk++;
    if (c->n3) {
        launch_pmat_fp64(c->d_pairs + c->n012, c->n3, h->d_label, h->d_tnode, c->d_prm3,
                         c->d_Pt + (size_t)c->n012 * 4096, h->stream);
        nk++;
    }
    const int H = (int)c->level_off.size() - 1;
    for (int L = 0; L < H; L++) {
        const int n = c->level_off[L + 1] - c->level_off[L];
        if (n == 0) continue;
        launch_prune_fp64(c->d_items + c->level_off[L], n, h->ntile, h->npad, h->d_z, c->d_Pt, c->d_conP, nullptr,
                          c->d_scaleF, c->d_scale_list, h->nscale, h->d_pi, h->d_fbar, h->d_ssum, h->d_fhK,
                          h->stream, h->d_amb);
        nk++;
    }
    cudaMemcpyAsync(h->d_fhK + (size_t)3 * h->npad, h->d_fhK + (size_t)2 * h->npad, sizeof(double) * h->npad,
                    cudaMemcpyDeviceToDevice, h->stream);
    launch_mix(h->d_fhK, h->d_fpatt, h->d_prm, h->npatt, h->npad, h->nscale, h->d_lnf, h->d_post, h->d_partial,
               h->d_ticket, h->d_out, h->stream);
    nk++;
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture (clade graph)");
    e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (clade graph)");
    c->kernels = nk;
    return 0;
}

// the clade schedule and graph, built on the handle's first clade evaluation
int clade_init(gb_handle *h) {
    if (h->clade) return 0;
    CladeState *c = new CladeState;
    const int rc = clade_setup(h, c);
    if (rc) {
        cudaStreamCaptureStatus cs;
        if (cudaStreamIsCapturing(h->stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(h->stream, &g);
            if (g) cudaGraphDestroy(g);
        }
        clade_free(c);
        return rc;
    }
    h->clade = c;
    return 0;
}

}  // namespace
}  // namespace gb

using namespace gb;

namespace {
// one evaluation from the four eigen solutions (host arrays), Qfactors, class weights
int eval_clade(gb_handle *h, const double *const U[4], const double *const V[4], const double *const Root[4],
               const double qfactor[2], const double freqK[3], const double *blength, double *neg_lnL, double *fhK,
               double *lnf, gb_stats *stats) {
    if (h->precision != GB_PREC_FP64) return fail(GB_ERR_ARG, "clade models: FP64 handles only");
    CK(cudaSetDevice(h->device));
    const double t0 = now_ms();
    for (int n = 0; n < h->nnode; n++) {
        const double t = n == h->root ? 0.0 : blength[n];
        if (!(t >= 0.0) || !std::isfinite(t)) return fail(GB_ERR_PARAM, "negative or non-finite branch length");
        h->h_tnode[n] = t;
    }
    int rc = clade_init(h);
    if (rc) return rc;
    CladeState *c = h->clade;
    DevParams *p = h->h_prm, *p3 = c->h_prm3;
    for (int i = 0; i < 3; i++) {
        std::memcpy(p->U[i], U[i], sizeof(double) * 61 * 61);
        std::memcpy(p->V[i], V[i], sizeof(double) * 61 * 61);
        std::memcpy(p->Root[i], Root[i], sizeof(double) * 61);
    }
    std::memcpy(p3->U[0], U[3], sizeof(double) * 61 * 61);
    std::memcpy(p3->V[0], V[3], sizeof(double) * 61 * 61);
    std::memcpy(p3->Root[0], Root[3], sizeof(double) * 61);
    std::memcpy(p->qf, qfactor, sizeof(double) * 2);
    std::memcpy(p3->qf, qfactor, sizeof(double) * 2);
    for (int k = 0; k < 3; k++) p->freqK[k] = freqK[k];
    p->freqK[3] = 0.0;
    p->sym = p3->sym = 0;
    CK(cudaEventRecord(h->ev0, h->stream));
    CK(cudaMemcpyAsync(h->d_prm, p, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(c->d_prm3, p3, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_tnode, h->h_tnode, sizeof(double) * h->nnode, cudaMemcpyHostToDevice, h->stream));
    CK(cudaGraphLaunch(c->graph, h->stream));
    CK(cudaMemcpyAsync(h->h_out, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (fhK)
        CK(cudaMemcpy2DAsync(fhK, sizeof(double) * h->npatt, h->d_fhK, sizeof(double) * h->npad,
                             sizeof(double) * h->npatt, 3, cudaMemcpyDeviceToHost, h->stream));
    if (lnf) CK(cudaMemcpyAsync(lnf, h->d_lnf, sizeof(double) * h->npatt, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    if (neg_lnL) *neg_lnL = h->h_out[0];
    h->kernels_last = c->kernels;
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        stats->ms_device = ms;
        stats->ms_host = now_ms() - t0;
        stats->kernels = c->kernels;
        stats->nscale = h->nscale;
        stats->h2d_bytes = 2 * sizeof(DevParams) + sizeof(double) * h->nnode;
        stats->d2h_bytes = sizeof(double) * (1 + (fhK ? 3 * h->npatt : 0) + (lnf ? h->npatt : 0));
    }
    return GB_OK;
}
}  // namespace

extern "C" int gb_eval_clade_uvr(gb_handle *h, const double *const U[4], const double *const V[4],
                                 const double *const Root[4], const double qfactor[2], const double freqK[3],
                                 const double *blength, double *neg_lnL, double *fhK, double *lnf,
                                 gb_stats *stats) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!U || !V || !Root || !qfactor || !freqK || !blength) return fail(GB_ERR_ARG, "null argument");
    for (int i = 0; i < 4; i++)
        if (!U[i] || !V[i] || !Root[i]) return fail(GB_ERR_ARG, "null U/V/Root");
    return eval_clade(h, U, V, Root, qfactor, freqK, blength, neg_lnL, fhK, lnf, stats);
}

// Clade models C / D from their parameters (SetParametersNSsites
// codeml.c:2522-2539): branch type b's Qfactor is 1 / meanrate(Q(kappa,
// p0 w0 + p1 w1 + p2 w_{2+b})) and the eigen solutions are those of Q(kappa,
// w) for w0, w1, w2, w3, from the library's host code.
extern "C" int gb_eval_clade(gb_handle *h, const double *blength, double kappa, double p0, double p1,
                             const double omega[4], double *neg_lnL, double *fhK, double *lnf, gb_stats *stats) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!blength || !omega) return fail(GB_ERR_ARG, "null argument");
    const double p2 = 1.0 - p0 - p1;
    if (!(kappa > 0.0) || !(p0 >= 0.0) || !(p1 >= 0.0) || !(p2 >= -1e-12) || !std::isfinite(kappa))
        return fail(GB_ERR_PARAM, "clade model parameters out of range");
    for (int i = 0; i < 4; i++)
        if (!(omega[i] >= 0.0) || !std::isfinite(omega[i])) return fail(GB_ERR_PARAM, "omega out of range");
    const double *pi = h->pi.data();
    std::vector<double> buf((size_t)4 * (2 * 61 * 61 + 61));
    double *U[4], *V[4], *R[4];
    for (int i = 0; i < 4; i++) {
        U[i] = buf.data() + (size_t)i * (2 * 61 * 61 + 61);
        V[i] = U[i] + 61 * 61;
        R[i] = V[i] + 61 * 61;
        std::vector<double> Q(61 * 61);
        build_q(pi, kappa, omega[i], Q.data(), nullptr, nullptr);
        if (eigen_qrev(Q.data(), pi, U[i], V[i], R[i])) return fail(GB_ERR_PARAM, "eigen solution failed");
    }
    const double fk[3] = {p0, p1, p2 > 0.0 ? p2 : 0.0};
    double qf[2];
    for (int b = 0; b < 2; b++) {
        std::vector<double> Q(61 * 61);
        qf[b] = 1.0 / build_q(pi, kappa, p0 * omega[0] + p1 * omega[1] + fk[2] * omega[2 + b], Q.data(), nullptr,
                              nullptr);
    }
    return eval_clade(h, U, V, R, qf, fk, blength, neg_lnL, fhK, lnf, stats);
}
