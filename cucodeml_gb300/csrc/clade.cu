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
//
// The gradient (gb_eval_clade with grad) is the FP64 adjoint of adjoint.cu
// run over this schedule: the forward keeps its edge messages, one backward
// item per (node, class) (no class shares a child's slot with another), the
// dlnL/dP partials of every pair, and the per-pair sums (dt', kappa, omega)
// against the parameter block that holds the pair's eigen solution; the chain
// rule through the branch types' Qfactors and the class weights on the host.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "adjoint_internal.h"
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
    std::vector<int> slot_of, sslot_of, pair_of;   // [nnode*3], [nnode*3], [nnode*4]
    // adjoint: backward items (top-down levels), dlnL/dP contributions per pair
    std::vector<BItem> bitems;
    std::vector<int> blevel_off, coff;
    std::vector<Contrib> contrib;
    int nchunk = 1, nfreq_blocks = 1;
    BItem *d_bitems = nullptr;
    Contrib *d_contrib = nullptr;
    int *d_coff = nullptr;
    double *d_E = nullptr, *d_Ebar = nullptr, *d_Abar = nullptr, *d_Gpart = nullptr;
    double *d_Dm = nullptr, *d_Dm3 = nullptr, *d_pout = nullptr, *d_fpart = nullptr;
    GradParams *d_gp = nullptr, *d_gp3 = nullptr, *h_gp = nullptr, *h_gp3 = nullptr;
    double *h_pout = nullptr, *h_fpart = nullptr;
    cudaGraphExec_t graph_g = nullptr;              // forward with edge messages, then the backward sweep
    int kernels_g = 0;
};

void clade_free(CladeState *c) {
    if (!c) return;
    if (c->graph) cudaGraphExecDestroy(c->graph);
    if (c->graph_g) cudaGraphExecDestroy(c->graph_g);
    void *dev[] = {c->d_items, c->d_pairs, c->d_scale_list, c->d_Pt, c->d_conP, c->d_scaleF, c->d_prm3,
                   c->d_bitems, c->d_contrib, c->d_coff, c->d_E, c->d_Ebar, c->d_Abar, c->d_Gpart,
                   c->d_Dm, c->d_Dm3, c->d_pout, c->d_fpart, c->d_gp, c->d_gp3};
    for (void *p : dev)
        if (p) cudaFree(p);
    void *host[] = {c->h_prm3, c->h_gp, c->h_gp3, c->h_pout, c->h_fpart};
    for (void *p : host)
        if (p) cudaFreeHost(p);
    delete c;
}

namespace {

// the three-class schedule over the handle's tree, heights and scaled nodes
void build_clade_schedule(const gb_handle *h, CladeState *c) {
    const int nn = h->nnode, ns = h->ns;
    std::vector<int> &slot_of = c->slot_of, &sslot_of = c->sslot_of, &pair_of = c->pair_of;
    slot_of.assign((size_t)nn * 3, -1);
    sslot_of.assign((size_t)nn * 3, -1);
    for (int a = ns; a < nn; a++)
        for (int k = 0; k < 3; k++) {
            slot_of[a * 3 + k] = c->nslot++;
            if (h->scale[a]) sslot_of[a * 3 + k] = c->nsslot++;
        }
    // eigen solution of class k on a branch of type lab: w0, w1, then w2 / w3
    auto wof = [](int k, int lab) { return k < 2 ? k : 2 + lab; };
    pair_of.assign((size_t)nn * 4, -1);
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

// one evaluation's forward on h->stream: P(t) of both parameter blocks, the
// pruning level by level (edge messages into E when given), class 3's fhK
// row from class 2's, the mixture; returns the kernel count
int record_clade_forward(gb_handle *h, CladeState *c, double *E) {
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
        launch_prune_fp64(c->d_items + c->level_off[L], n, h->ntile, h->npad, h->d_z, c->d_Pt, c->d_conP, E,
                          c->d_scaleF, c->d_scale_list, h->nscale, h->d_pi, h->d_fbar, h->d_ssum, h->d_fhK,
                          h->stream, h->d_amb);
        nk++;
    }
    cudaMemcpyAsync(h->d_fhK + (size_t)3 * h->npad, h->d_fhK + (size_t)2 * h->npad, sizeof(double) * h->npad,
                    cudaMemcpyDeviceToDevice, h->stream);
    launch_mix(h->d_fhK, h->d_fpatt, h->d_prm, h->npatt, h->npad, h->nscale, h->d_lnf, h->d_post, h->d_partial,
               h->d_ticket, h->d_out, h->stream);
    return nk + 1;
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
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const int nk = record_clade_forward(h, c, nullptr);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture (clade graph)");
    e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (clade graph)");
    c->kernels = nk;
    return 0;
}

// The adjoint's structures: one backward item per (node, class), levels from
// the root down; each pair's dlnL/dP contributions (parent slot's edge row,
// child slot or tip); buffers; one graph of the forward with edge messages
// and the backward sweep.
int clade_grad_setup(gb_handle *h, CladeState *c) {
    const int ns = h->ns, nn = h->nnode, H = h->height[h->root];
    auto wof = [](int k, int lab) { return k < 2 ? k : 2 + lab; };
    for (int L = H; L >= 1; L--) {
        c->blevel_off.push_back((int)c->bitems.size());
        for (int n = ns; n < nn; n++) {
            if (h->height[n] != L) continue;
            for (int k = 0; k < 3; k++) {
                BItem b{};
                b.node = n;
                b.is_root = n == h->root;
                b.nchild = h->nson[n];
                b.ncls = 1;
                b.cls[0] = b.cls[1] = k;
                b.pslot[0] = c->slot_of[n * 3 + k];
                b.pslot[1] = -1;
                b.sslot[0] = h->scale[n] ? c->sslot_of[n * 3 + k] : -1;
                b.sslot[1] = -1;
                b.eslot[0] = b.pslot[0] * MAXC;
                b.eslot[1] = -1;
                for (int i = 0; i < MAXC; i++) {
                    b.child[i] = -1;
                    b.pidx[i][0] = b.pidx[i][1] = b.tslot[i][0] = b.tslot[i][1] = -1;
                }
                for (int i = 0; i < b.nchild; i++) {
                    const int sn = h->sons[n * MAXC + i];
                    b.child[i] = sn;
                    b.pidx[i][0] = b.pidx[i][1] = c->pair_of[sn * 4 + wof(k, h->label[sn])];
                    b.tslot[i][0] = b.tslot[i][1] = sn < ns ? -1 : c->slot_of[sn * 3 + k];
                }
                c->bitems.push_back(b);
            }
        }
    }
    c->blevel_off.push_back((int)c->bitems.size());
    const size_t npair = c->pairs.size();
    std::vector<std::vector<Contrib>> per(npair);
    for (const Item &it : c->items)
        for (int i = 0; i < it.nchild; i++) per[it.pidx[i]].push_back(Contrib{it.eslot + i, it.cslot[i], it.child[i]});
    c->coff.assign(npair + 1, 0);
    for (size_t p = 0; p < npair; p++) {
        c->coff[p + 1] = c->coff[p] + (int)per[p].size();
        for (const Contrib &cb : per[p]) c->contrib.push_back(cb);
    }
    c->nchunk = (h->npatt + GCHUNK - 1) / GCHUNK;
    c->nfreq_blocks = (h->npatt + 255) / 256;
    const size_t npad = h->npad, erows = (size_t)c->nslot * MAXC * npad * 64;
    int rc;
    if ((rc = dalloc(&c->d_bitems, c->bitems.size())) || (rc = dalloc(&c->d_contrib, c->contrib.size())) ||
        (rc = dalloc(&c->d_coff, c->coff.size())) || (rc = dalloc(&c->d_E, erows)) ||
        (rc = dalloc(&c->d_Ebar, erows)) || (rc = dalloc(&c->d_Abar, (size_t)c->nslot * npad * 64)) ||
        (rc = dalloc(&c->d_Gpart, npair * c->nchunk * 64 * 64)) || (rc = dalloc(&c->d_Dm, DM_MATS * 64 * 64)) ||
        (rc = dalloc(&c->d_Dm3, DM_MATS * 64 * 64)) || (rc = dalloc(&c->d_pout, npair * 3)) ||
        (rc = dalloc(&c->d_fpart, (size_t)c->nfreq_blocks * 4)) || (rc = dalloc(&c->d_gp, 1)) ||
        (rc = dalloc(&c->d_gp3, 1)))
        return rc;
    if (cudaMallocHost((void **)&c->h_gp, sizeof(GradParams)) || cudaMallocHost((void **)&c->h_gp3, sizeof(GradParams)) ||
        cudaMallocHost((void **)&c->h_pout, sizeof(double) * npair * 3) ||
        cudaMallocHost((void **)&c->h_fpart, sizeof(double) * c->nfreq_blocks * 4))
        return fail(GB_ERR_OOM, "cudaMallocHost (clade adjoint)");
    std::memset(c->h_gp, 0, sizeof(GradParams));
    std::memset(c->h_gp3, 0, sizeof(GradParams));
    CK(cudaMemcpy(c->d_bitems, c->bitems.data(), sizeof(BItem) * c->bitems.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_contrib, c->contrib.data(), sizeof(Contrib) * c->contrib.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->d_coff, c->coff.data(), sizeof(int) * c->coff.size(), cudaMemcpyHostToDevice));
    // padded patterns keep zero upper partials (their seed has fpatt = 0)
    CK(cudaMemset(c->d_Abar, 0, sizeof(double) * (size_t)c->nslot * npad * 64));
    CK(init_fp64_adjoint_kernels());
    cudaStream_t st = h->stream;
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    int nk = record_clade_forward(h, c, c->d_E);
    launch_dmat_fp64(h->d_prm, c->d_gp, c->d_Dm, st);
    nk++;
    if (c->n3) {
        launch_dmat_fp64(c->d_prm3, c->d_gp3, c->d_Dm3, st);
        nk++;
    }
    for (size_t L = 0; L + 1 < c->blevel_off.size(); L++) {
        const int n = c->blevel_off[L + 1] - c->blevel_off[L];
        if (!n) continue;
        launch_bwd_level_fp64(c->d_bitems + c->blevel_off[L], n, h->ntile, h->npad, c->d_Pt, c->d_E, c->d_Ebar,
                              c->d_Abar, c->d_scaleF, h->d_fpatt, h->d_post, h->d_fbar, h->d_pi, st);
        nk++;
    }
    launch_gradP_fp64(c->d_contrib, c->d_coff, (int)npair, c->nchunk, h->npatt, h->npad, c->d_Ebar, c->d_conP,
                      h->d_z, c->d_Gpart, h->d_amb, st);
    nk++;
    launch_gradH_fp64(c->d_pairs, c->n012, h->d_label, h->d_tnode, h->d_prm, c->d_Gpart, c->nchunk, c->d_Dm,
                      c->d_pout, st);
    nk++;
    if (c->n3) {
        launch_gradH_fp64(c->d_pairs + c->n012, c->n3, h->d_label, h->d_tnode, c->d_prm3,
                          c->d_Gpart + (size_t)c->n012 * c->nchunk * 64 * 64, c->nchunk, c->d_Dm3,
                          c->d_pout + (size_t)c->n012 * 3, st);
        nk++;
    }
    launch_freq_fp64(h->d_fhK, h->d_lnf, h->d_fpatt, h->npatt, h->npad, h->nscale, c->d_fpart, st);
    nk++;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture (clade gradient graph)");
    e = cudaGraphInstantiate(&c->graph_g, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (clade gradient graph)");
    c->kernels_g = nk;
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

// the adjoint's structures and graph, on the first clade gradient
int clade_grad_init(gb_handle *h) {
    CladeState *c = h->clade;
    if (c->graph_g) return 0;
    const int rc = clade_grad_setup(h, c);
    if (rc) {
        cudaStreamCaptureStatus cs;
        if (cudaStreamIsCapturing(h->stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(h->stream, &g);
            if (g) cudaGraphDestroy(g);
        }
        // the next clade call sets the whole state up again
        h->clade = nullptr;
        clade_free(c);
        return rc;
    }
    return 0;
}

}  // namespace
}  // namespace gb

using namespace gb;

namespace {
// one evaluation from the four eigen solutions (host arrays), Qfactors and
// class weights; with gp / gp3 (the dQ/dkappa, dQ/domega of the two parameter
// blocks) also the adjoint, its per-pair and class-weight sums left in
// h->clade->h_pout / h_fpart
int eval_clade(gb_handle *h, const double *const U[4], const double *const V[4], const double *const Root[4],
               const double qfactor[2], const double freqK[3], const double *blength, const GradParams *gp,
               const GradParams *gp3, double *neg_lnL, double *fhK, double *lnf, gb_stats *stats) {
    if (h->precision != GB_PREC_FP64) return fail(GB_ERR_ARG, "clade models: FP64 handles only");
    CK(cudaSetDevice(h->device));
    const double t0 = now_ms();
    for (int n = 0; n < h->nnode; n++) {
        const double t = n == h->root ? 0.0 : blength[n];
        if (!(t >= 0.0) || !std::isfinite(t)) return fail(GB_ERR_PARAM, "negative or non-finite branch length");
        h->h_tnode[n] = t;
    }
    int rc = clade_init(h);
    if (!rc && gp) rc = clade_grad_init(h);
    if (rc) return rc;
    CladeState *c = h->clade;
    DevParams *p = h->h_prm, *p3 = c->h_prm3;
    for (int i = 0; i < 3; i++) {
        std::memcpy(p->U[i], U[i], sizeof(double) * 61 * 61);
        std::memcpy(p->V[i], V[i], sizeof(double) * 61 * 61);
        std::memcpy(p->Root[i], Root[i], sizeof(double) * 61);
        // the second block holds solution 3 in every slot (only slot 0 is read by a pair)
        std::memcpy(p3->U[i], U[3], sizeof(double) * 61 * 61);
        std::memcpy(p3->V[i], V[3], sizeof(double) * 61 * 61);
        std::memcpy(p3->Root[i], Root[3], sizeof(double) * 61);
    }
    std::memcpy(p->qf, qfactor, sizeof(double) * 2);
    std::memcpy(p3->qf, qfactor, sizeof(double) * 2);
    for (int k = 0; k < 3; k++) p->freqK[k] = freqK[k];
    p->freqK[3] = 0.0;
    p->sym = p3->sym = 0;
    const size_t npair = c->pairs.size();
    CK(cudaEventRecord(h->ev0, h->stream));
    CK(cudaMemcpyAsync(h->d_prm, p, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(c->d_prm3, p3, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_tnode, h->h_tnode, sizeof(double) * h->nnode, cudaMemcpyHostToDevice, h->stream));
    if (gp) {
        std::memcpy(c->h_gp, gp, sizeof(GradParams));
        std::memcpy(c->h_gp3, gp3, sizeof(GradParams));
        CK(cudaMemcpyAsync(c->d_gp, c->h_gp, sizeof(GradParams), cudaMemcpyHostToDevice, h->stream));
        CK(cudaMemcpyAsync(c->d_gp3, c->h_gp3, sizeof(GradParams), cudaMemcpyHostToDevice, h->stream));
        CK(cudaGraphLaunch(c->graph_g, h->stream));
        CK(cudaMemcpyAsync(c->h_pout, c->d_pout, sizeof(double) * npair * 3, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaMemcpyAsync(c->h_fpart, c->d_fpart, sizeof(double) * c->nfreq_blocks * 4, cudaMemcpyDeviceToHost,
                           h->stream));
    } else {
        CK(cudaGraphLaunch(c->graph, h->stream));
    }
    CK(cudaMemcpyAsync(h->h_out, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (fhK)
        CK(cudaMemcpy2DAsync(fhK, sizeof(double) * h->npatt, h->d_fhK, sizeof(double) * h->npad,
                             sizeof(double) * h->npatt, 3, cudaMemcpyDeviceToHost, h->stream));
    if (lnf) CK(cudaMemcpyAsync(lnf, h->d_lnf, sizeof(double) * h->npatt, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    if (neg_lnL) *neg_lnL = h->h_out[0];
    h->kernels_last = gp ? c->kernels_g : c->kernels;
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        stats->ms_device = ms;
        stats->ms_host = now_ms() - t0;
        stats->kernels = h->kernels_last;
        stats->nscale = h->nscale;
        stats->h2d_bytes = 2 * sizeof(DevParams) + sizeof(double) * h->nnode + (gp ? 2 * sizeof(GradParams) : 0);
        stats->d2h_bytes = sizeof(double) * (1 + (fhK ? 3 * h->npatt : 0) + (lnf ? h->npatt : 0) +
                                             (gp ? npair * 3 + c->nfreq_blocks * 4 : 0));
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
    return eval_clade(h, U, V, Root, qfactor, freqK, blength, nullptr, nullptr, neg_lnL, fhK, lnf, stats);
}

// Clade models C / D from their parameters (SetParametersNSsites
// codeml.c:2522-2539): branch type b's Qfactor is 1 / meanrate(Q(kappa,
// wbar_b)), wbar_b = p0 w0 + p1 w1 + p2 w_{2+b}, and the eigen solutions are
// those of Q(kappa, w) for w0, w1, w2, w3, from the library's host code.  The
// gradient's chain rule: dlnL/dt = dlnL/dt' qf_b; the Qfactors through
// dmr/dkappa = part1 + wbar part3 and dmr/dwbar = part2 + kappa part3 (mr =
// part0 + kappa part1 + wbar part2 + kappa wbar part3); the class weights
// (p0, p1, 1 - p0 - p1) through the mixture's sums.
extern "C" int gb_eval_clade(gb_handle *h, const double *blength, double kappa, double p0, double p1,
                             const double omega[4], double *neg_lnL, double *grad, double *fhK, double *lnf,
                             gb_stats *stats) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!blength || !omega) return fail(GB_ERR_ARG, "null argument");
    const double p2 = 1.0 - p0 - p1;
    if (!(kappa > 0.0) || !(p0 >= 0.0) || !(p1 >= 0.0) || !(p2 >= -1e-12) || !std::isfinite(kappa))
        return fail(GB_ERR_PARAM, "clade model parameters out of range");
    for (int i = 0; i < 4; i++)
        if (!(omega[i] >= 0.0) || !std::isfinite(omega[i])) return fail(GB_ERR_PARAM, "omega out of range");
    const double *pi = h->pi.data();
    const int NQ = 61 * 61;
    std::vector<double> buf((size_t)4 * (2 * NQ + 61)), Q(NQ);
    std::vector<GradParams> gps(grad ? 2 : 0);
    double *U[4], *V[4], *R[4];
    for (int i = 0; i < 4; i++) {
        U[i] = buf.data() + (size_t)i * (2 * NQ + 61);
        V[i] = U[i] + NQ;
        R[i] = V[i] + NQ;
        GradParams *g = grad ? &gps[i < 3 ? 0 : 1] : nullptr;
        const int slot = i < 3 ? i : 0;
        build_q(pi, kappa, omega[i], Q.data(), g ? g->dQk[slot] : nullptr, g ? g->dQw[slot] : nullptr);
        if (eigen_qrev(Q.data(), pi, U[i], V[i], R[i])) return fail(GB_ERR_PARAM, "eigen solution failed");
    }
    if (grad)
        for (int i = 1; i < 3; i++) {       // the second block's unused slots repeat solution 3
            std::memcpy(gps[1].dQk[i], gps[1].dQk[0], sizeof(double) * NQ);
            std::memcpy(gps[1].dQw[i], gps[1].dQw[0], sizeof(double) * NQ);
        }
    const double fk[3] = {p0, p1, p2 > 0.0 ? p2 : 0.0};
    double qf[2], wbar[2];
    for (int b = 0; b < 2; b++) {
        wbar[b] = p0 * omega[0] + p1 * omega[1] + fk[2] * omega[2 + b];
        qf[b] = 1.0 / build_q(pi, kappa, wbar[b], Q.data(), nullptr, nullptr);
    }
    const int rc = eval_clade(h, U, V, R, qf, fk, blength, grad ? &gps[0] : nullptr, grad ? &gps[1] : nullptr,
                              neg_lnL, fhK, lnf, stats);
    if (rc || !grad) return rc;
    // chain rule on the host (derivatives of lnL, negated at the end)
    const CladeState *c = h->clade;
    const int nn = h->nnode;
    std::vector<double> dtp(nn, 0.0);
    double dk = 0.0, dom[4] = {0, 0, 0, 0};
    for (size_t q = 0; q < c->pairs.size(); q++) {
        const PairDesc &pd = c->pairs[q];
        dtp[pd.node] += c->h_pout[q * 3 + 0];
        dk += c->h_pout[q * 3 + 1];
        dom[(int)q < c->n012 ? pd.w : 3] += c->h_pout[q * 3 + 2];
    }
    double dqf[2] = {0, 0};
    for (int n = 0; n < nn; n++) {
        if (n == h->root) {
            grad[n] = 0.0;
            continue;
        }
        const int b = h->label[n];
        grad[n] = -dtp[n] * qf[b];
        dqf[b] += dtp[n] * blength[n];
    }
    double dfk[3] = {0, 0, 0};
    for (int q = 0; q < c->nfreq_blocks; q++)
        for (int k = 0; k < 3; k++) dfk[k] += c->h_fpart[q * 4 + k];
    double part[4];
    mean_rate_parts(pi, part);
    double gk = dk, gw[4] = {dom[0], dom[1], dom[2], dom[3]};
    double gp0 = dfk[0] - dfk[2], gp1 = dfk[1] - dfk[2];
    for (int b = 0; b < 2; b++) {
        const double q2 = -qf[b] * qf[b];
        gk += dqf[b] * q2 * (part[1] + wbar[b] * part[3]);
        const double gwb = dqf[b] * q2 * (part[2] + kappa * part[3]);    // dlnL/dwbar_b
        gw[0] += gwb * p0;
        gw[1] += gwb * p1;
        gw[2 + b] += gwb * fk[2];
        gp0 += gwb * (omega[0] - omega[2 + b]);
        gp1 += gwb * (omega[1] - omega[2 + b]);
    }
    grad[nn + 0] = -gk;
    grad[nn + 1] = -gp0;
    grad[nn + 2] = -gp1;
    for (int i = 0; i < 4; i++) grad[nn + 3 + i] = -gw[i];
    return GB_OK;
}

// gb_eval_clade in codeml's x space (branch lengths in codeml's branch order,
// kappa, p0, p1 -- transformed unless lastround, as f_and_x does -- then w0,
// [w1 under model D], w2, w3); f = -lnL, dx its gradient.
extern "C" int gb_dfun_clade_x(gb_handle *h, const int *bnode, int lastround, int model_d, const double *x, int n,
                               double *f, double *dx) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    const int nb = h->nnode - 1;
    if (!bnode || !x || !f || !dx || n != nb + (model_d ? 7 : 6)) return fail(GB_ERR_ARG, "gb_dfun_clade_x: bad arguments");
    std::vector<double> bl(h->nnode, 0.0), g(h->nnode + 7, 0.0);
    for (int ib = 0; ib < nb; ib++) {
        if (bnode[ib] < 0 || bnode[ib] >= h->nnode || bnode[ib] == h->root) return fail(GB_ERR_ARG, "bnode");
        bl[bnode[ib]] = x[ib];
    }
    double p0 = x[nb + 1], p1 = x[nb + 2];
    if (!lastround) {       // p_i = e^{x_i} / (1 + e^{x_1} + e^{x_2})
        const double e1 = std::exp(x[nb + 1]), e2 = std::exp(x[nb + 2]), tot = 1 + e1 + e2;
        p0 = e1 / tot;
        p1 = e2 / tot;
    }
    const double om[4] = {x[nb + 3], model_d ? x[nb + 4] : 1.0, x[n - 2], x[n - 1]};
    const int rc = gb_eval_clade(h, bl.data(), x[nb], p0, p1, om, f, g.data(), nullptr, nullptr, nullptr);
    if (rc) return rc;
    const int nn = h->nnode;
    for (int ib = 0; ib < nb; ib++) dx[ib] = g[bnode[ib]];
    dx[nb] = g[nn];
    const double gp0 = g[nn + 1], gp1 = g[nn + 2];
    if (!lastround) {
        dx[nb + 1] = gp0 * p0 * (1 - p0) - gp1 * p0 * p1;
        dx[nb + 2] = -gp0 * p0 * p1 + gp1 * p1 * (1 - p1);
    } else {
        dx[nb + 1] = gp0;
        dx[nb + 2] = gp1;
    }
    dx[nb + 3] = g[nn + 3];
    if (model_d) dx[nb + 4] = g[nn + 4];
    dx[n - 2] = g[nn + 5];
    dx[n - 1] = g[nn + 6];
    return GB_OK;
}

// codeml's NEB under the clade models (lfunNSsites_rate codeml.c:5079-5129:
// freqK_c f_c / sum over the three classes at the parameters): the mixture
// kernel's class posteriors of one gb_eval_clade evaluation, [3][npatt].
extern "C" int gb_neb_clade(gb_handle *h, const double *blength, double kappa, double p0, double p1,
                            const double omega[4], double *post, double *neg_lnL) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!post) return fail(GB_ERR_ARG, "null argument");
    const int rc = gb_eval_clade(h, blength, kappa, p0, p1, omega, neg_lnL, nullptr, nullptr, nullptr, nullptr);
    if (rc) return rc;
    CK(cudaMemcpy2D(post, sizeof(double) * h->npatt, h->d_post, sizeof(double) * h->npad,
                    sizeof(double) * h->npatt, 3, cudaMemcpyDeviceToHost));
    return GB_OK;
}
