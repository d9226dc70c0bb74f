// Host runtime and C ABI of libgbcodeml.so (see include/gbcodeml.h).
//
// gb_create builds a level schedule of the tree once (replacing the BFS layer
// schedule and per-node streams of prepareTree / schedule,
// cuda-codeml.cu:851-919, 1280-1334): internal nodes are grouped by height,
// and each level is ONE kernel launch over every (node, class, pattern tile)
// of that level, so an evaluation is 1 + H + 1 launches (H = tree height)
// instead of ~520 launches and ~250 host syncs per lnL.  The launches of an
// evaluation are captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gbcodeml.h"
#include "internal.h"
#include "model.h"
#include "handle.h"
#include "adjoint_internal.h"

using namespace gb;

namespace gb {

namespace {
thread_local std::string g_err;
}

int fail(int code, const std::string &msg) {
    g_err = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(e == cudaErrorMemoryAllocation ? GB_ERR_OOM : GB_ERR_CUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

}  // namespace gb

namespace {

int build_schedule(gb_handle *h, const gb_problem *p) {
    const int nn = p->nnode, ns = p->ns;
    if (ns < 3 || nn < ns + 1 || p->npatt < 1 || !p->father || !p->label || !p->z || !p->fpatt || !p->pi)
        return fail(GB_ERR_ARG, "gb_problem: missing arrays or sizes too small");
    if (p->root < ns || p->root >= nn || p->father[p->root] != -1)
        return fail(GB_ERR_ARG, "gb_problem: root must be an internal node with father -1");
    h->ns = ns; h->nnode = nn; h->root = p->root; h->npatt = p->npatt;
    // pattern padding: 32-pattern tiles (FP64) or 128-pattern tiles (split precision)
    const int unit = h->precision == GB_PREC_FP64 ? TILE64 : 128;
    h->npad = (p->npatt + unit - 1) / unit * unit;
    h->ntile = h->npad / TILE64;
    h->father.assign(p->father, p->father + nn);
    h->label.assign(nn, 0);
    h->nson.assign(nn, 0);
    h->sons.assign((size_t)nn * MAXC, -1);
    for (int n = 0; n < nn; n++) {
        if (n == p->root) continue;
        int f = p->father[n];
        if (f < ns || f >= nn) return fail(GB_ERR_ARG, "gb_problem: father out of range or a tip");
        if (h->nson[f] >= MAXC) return fail(GB_ERR_ARG, "gb_problem: more than 3 sons at a node");
        h->sons[f * MAXC + h->nson[f]++] = n;
        int lab = p->label[n];
        if (lab != 0 && lab != 1) return fail(GB_ERR_ARG, "gb_problem: branch labels must be 0 or 1");
        h->label[n] = lab;
    }
    for (int n = 0; n < nn; n++) {
        if (n < ns && h->nson[n] != 0) return fail(GB_ERR_ARG, "gb_problem: tips must be nodes 0..ns-1");
        if (n >= ns && h->nson[n] < 2) return fail(GB_ERR_ARG, "gb_problem: internal node with < 2 sons");
    }
    // heights (post-order by repeated relaxation over a reverse BFS order)
    std::vector<int> order;
    order.push_back(h->root);
    for (size_t i = 0; i < order.size(); i++)
        for (int k = 0; k < h->nson[order[i]]; k++) order.push_back(h->sons[order[i] * MAXC + k]);
    if ((int)order.size() != nn) return fail(GB_ERR_ARG, "gb_problem: tree is not connected");
    h->height.assign(nn, 0);
    h->dirty.assign(nn, 0);
    for (int i = nn - 1; i >= 0; i--) {
        int a = order[i];
        for (int k = 0; k < h->nson[a]; k++) {
            int s = h->sons[a * MAXC + k];
            h->height[a] = std::max(h->height[a], h->height[s] + 1);
            if (h->label[s] == 1 || h->dirty[s]) h->dirty[a] = 1;
        }
    }
    // scaled nodes: given, or codeml's rule (a node is scaled when more than
    // 15 tips hang below it since the last scaled node; never the root)
    h->scale.assign(nn, 0);
    if (p->node_scale) {
        for (int n = ns; n < nn; n++) h->scale[n] = p->node_scale[n] ? 1 : 0;
        h->scale[h->root] = 0;
    } else {
        std::vector<int> d(nn, 0);
        for (int i = nn - 1; i >= 0; i--) {
            int a = order[i];
            if (a < ns) { d[a] = 1; continue; }
            int s = 0;
            for (int k = 0; k < h->nson[a]; k++) s += d[h->sons[a * MAXC + k]];
            if (a != h->root && s > 15) {
                h->scale[a] = 1;
                s = 1;
            }
            d[a] = s;
        }
    }
    h->nscale = 0;
    for (int n = 0; n < nn; n++) h->nscale += h->scale[n];

    // slots: classes 0,1 everywhere; 2,3 at dirty nodes and the root
    h->slot_of.assign((size_t)nn * 4, -1);
    h->sslot_of.assign((size_t)nn * 4, -1);
    h->nslot = h->nsslot = 0;
    auto ncls = [&](int a) { return (h->dirty[a] || a == h->root) ? 4 : 2; };
    for (int a = ns; a < nn; a++)
        for (int c = 0; c < ncls(a); c++) {
            h->slot_of[a * 4 + c] = h->nslot++;
            if (h->scale[a]) h->sslot_of[a * 4 + c] = h->nsslot++;
        }
    auto cls_of = [&](int s, int c) { return (h->dirty[s] || s == h->root) ? c : (c & 1); };
    // transition matrices: w0 and w1 for every branch, w2 as well on foreground branches
    h->pair_of.assign((size_t)nn * 3, -1);
    h->pairs.clear();
    for (int n = 0; n < nn; n++) {
        if (n == h->root) continue;
        for (int w = 0; w < (h->label[n] ? 3 : 2); w++) {
            h->pair_of[n * 3 + w] = (int)h->pairs.size();
            h->pairs.push_back(PairDesc{n, w});
        }
    }
    h->scale_list.assign((size_t)4 * std::max(h->nscale, 1), 0);
    for (int c = 0; c < 4; c++) {
        int k = 0;
        for (int b = 0; b < nn; b++)
            if (h->scale[b]) h->scale_list[c * h->nscale + k++] = h->sslot_of[b * 4 + cls_of(b, c)];
    }
    // items by level
    int H = h->height[h->root];
    h->items.clear();
    h->level_off.assign(H + 1, 0);
    for (int L = 1; L <= H; L++) {
        h->level_off[L - 1] = (int)h->items.size();
        for (int a = ns; a < nn; a++) {
            if (h->height[a] != L) continue;
            for (int c = 0; c < ncls(a); c++) {
                Item it{};
                it.node = a; it.cls = c; it.slot = h->slot_of[a * 4 + c];
                it.nchild = h->nson[a];
                for (int k = 0; k < MAXC; k++) { it.child[k] = -1; it.cslot[k] = -1; it.pidx[k] = -1; }
                for (int k = 0; k < it.nchild; k++) {
                    int s = h->sons[a * MAXC + k];
                    it.child[k] = s;
                    it.cslot[k] = s < ns ? -1 : h->slot_of[s * 4 + cls_of(s, c)];
                    int w = h->label[s] == 0 ? (c & 1) : (c <= 1 ? c : 2);
                    it.pidx[k] = h->pair_of[s * 3 + w];
                }
                it.sslot = h->scale[a] ? h->sslot_of[a * 4 + c] : -1;
                it.is_root = a == h->root;
                it.eslot = it.slot * MAXC;
                h->items.push_back(it);
            }
        }
    }
    h->level_off[H] = (int)h->items.size();
    return 0;
}

void free_all(gb_handle *h) {
    if (!h) return;
    if (h->device >= 0) cudaSetDevice(h->device);
    for (auto &g : h->graph)
        if (g) cudaGraphExecDestroy(g);
    for (int m = 0; m < 16; m++) {
        if (h->graph_cls[m]) cudaGraphExecDestroy(h->graph_cls[m]);
        if (h->d_items_cls[m]) cudaFree(h->d_items_cls[m]);
    }
    void *dev[] = {h->d_items, h->d_pairs, h->d_label, h->d_scale_list, h->d_z, h->d_fpatt, h->d_pi,
                   h->d_tnode, h->d_prm, h->d_Pt, h->d_conP, h->d_E, h->d_scaleF, h->d_fbar,
                   h->d_ssum, h->d_fhK, h->d_lnf, h->d_post, h->d_partial, h->d_out, h->d_ticket,
                   h->d_amb};
    for (void *p : dev)
        if (p) cudaFree(p);
    if (h->h_prm) cudaFreeHost(h->h_prm);
    if (h->h_tnode) cudaFreeHost(h->h_tnode);
    if (h->h_out) cudaFreeHost(h->h_out);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    adjoint_free(h->adj);
    fast_free(h->fast);
    clade_free(h->clade);
    delete h;
}

// record the forward launches on h->stream; returns the number of kernels
int record_forward(gb_handle *h, bool keepE) {
    int nk = 0;
    launch_pmat_fp64(h->d_pairs, (int)h->pairs.size(), h->d_label, h->d_tnode, h->d_prm, h->d_Pt, h->stream,
                     h->d_pi);
    prof_mark(h, GB_K_PMAT);
    nk++;
    int H = (int)h->level_off.size() - 1;
    for (int L = 0; L < H; L++) {
        int n = h->level_off[L + 1] - h->level_off[L];
        if (n == 0) continue;
        launch_prune_fp64(h->d_items + h->level_off[L], n, h->ntile, h->npad, h->d_z, h->d_Pt,
                          h->d_conP, keepE ? h->d_E : nullptr, h->d_scaleF, h->d_scale_list,
                          h->nscale, h->d_pi, h->d_fbar, h->d_ssum, h->d_fhK, h->stream, h->d_amb);
        prof_mark(h, GB_K_PRUNE);
        nk++;
    }
    launch_mix(h->d_fhK, h->d_fpatt, h->d_prm, h->npatt, h->npad, h->nscale, h->d_lnf, h->d_post,
               h->d_partial, h->d_ticket, h->d_out, h->stream);
    prof_mark(h, GB_K_MIX);
    nk++;
    return nk;
}

int ensure_graph(gb_handle *h, bool keepE) {
    cudaGraphExec_t &ge = h->graph[keepE ? 1 : 0];
    if (ge) return 0;
    if (keepE && !h->d_E) {
        int rc = dalloc(&h->d_E, (size_t)h->nslot * MAXC * h->npad * 64);
        if (rc) return rc;
    }
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    h->graph_kernels = record_forward(h, keepE);
    CK(cudaStreamEndCapture(h->stream, &g));
    cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(GB_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return 0;
}

int upload_and_run(gb_handle *h, const Derived *D, const double *blength, bool keepE, double *neg_lnL,
                   double *fhK, double *lnf, gb_stats *stats) {
    CK(cudaSetDevice(h->device));
    double t0 = now_ms();
    for (int i = 0; i < 3; i++) {
        std::memcpy(h->h_prm->U[i], D->U[i], sizeof(double) * 61 * 61);
        std::memcpy(h->h_prm->V[i], D->V[i], sizeof(double) * 61 * 61);
        std::memcpy(h->h_prm->Root[i], D->Root[i], sizeof(double) * 61);
    }
    std::memcpy(h->h_prm->qf, D->qf, sizeof(double) * 2);
    std::memcpy(h->h_prm->freqK, D->freqK, sizeof(double) * 4);
    h->h_prm->sym = D->sym;
    for (int n = 0; n < h->nnode; n++) {
        double t = n == h->root ? 0.0 : blength[n];
        if (!(t >= 0.0) || !std::isfinite(t)) return fail(GB_ERR_PARAM, "negative or non-finite branch length");
        h->h_tnode[n] = t;
    }
    int rc = ensure_graph(h, keepE);
    if (rc) return rc;
    CK(cudaEventRecord(h->ev0, h->stream));
    CK(cudaMemcpyAsync(h->d_prm, h->h_prm, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_tnode, h->h_tnode, sizeof(double) * h->nnode, cudaMemcpyHostToDevice, h->stream));
    CK(cudaGraphLaunch(h->graph[keepE ? 1 : 0], h->stream));
    CK(cudaMemcpyAsync(h->h_out, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (fhK)
        CK(cudaMemcpy2DAsync(fhK, sizeof(double) * h->npatt, h->d_fhK, sizeof(double) * h->npad,
                             sizeof(double) * h->npatt, 4, cudaMemcpyDeviceToHost, h->stream));
    if (lnf) CK(cudaMemcpyAsync(lnf, h->d_lnf, sizeof(double) * h->npatt, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    *neg_lnL = h->h_out[0];
    h->kernels_last = h->graph_kernels;
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        stats->ms_device = ms;
        stats->ms_host = now_ms() - t0;
        stats->kernels = h->graph_kernels;
        stats->nscale = h->nscale;
        stats->h2d_bytes = sizeof(DevParams) + sizeof(double) * h->nnode;
        stats->d2h_bytes = sizeof(double) * (1 + (fhK ? 4 * h->npatt : 0) + (lnf ? h->npatt : 0));
    }
    return 0;
}

}  // namespace

namespace gb {
int stage_params(gb_handle *h, const Derived *D, const double *blength) {
    for (int i = 0; i < 3; i++) {
        std::memcpy(h->h_prm->U[i], D->U[i], sizeof(double) * 61 * 61);
        std::memcpy(h->h_prm->V[i], D->V[i], sizeof(double) * 61 * 61);
        std::memcpy(h->h_prm->Root[i], D->Root[i], sizeof(double) * 61);
    }
    std::memcpy(h->h_prm->qf, D->qf, sizeof(double) * 2);
    std::memcpy(h->h_prm->freqK, D->freqK, sizeof(double) * 4);
    h->h_prm->sym = D->sym;
    for (int n = 0; n < h->nnode; n++) {
        double t = n == h->root ? 0.0 : blength[n];
        if (!(t >= 0.0) || !std::isfinite(t)) return fail(GB_ERR_PARAM, "negative or non-finite branch length");
        h->h_tnode[n] = t;
    }
    return 0;
}

int fp64_prepare(gb_handle *h, bool grad) {
    CK(cudaSetDevice(h->device));
    int rc = ensure_graph(h, grad);          // allocates the edge messages when grad
    if (!rc && grad) rc = adjoint_init(h);
    return rc;
}

// the device work of one FP64 evaluation on h->stream (for batch graphs):
// parameter upload, forward, optional adjoint, result download
int fp64_record_eval(gb_handle *h, bool grad) {
    CK(cudaMemcpyAsync(h->d_prm, h->h_prm, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_tnode, h->h_tnode, sizeof(double) * h->nnode, cudaMemcpyHostToDevice, h->stream));
    int nk = record_forward(h, grad);
    if (grad) {
        CK(cudaMemcpyAsync(h->adj->d_gp, h->adj->h_gp, sizeof(GradParams), cudaMemcpyHostToDevice, h->stream));
        nk += adjoint_record(h);
        int rc = adjoint_fetch(h);
        if (rc) return rc;
    }
    CK(cudaMemcpyAsync(h->h_out, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    return nk;
}

void prof_mark(gb_handle *h, int cls) {
    if (!h->prof) return;
    cudaEvent_t e;
    cudaEventCreate(&e);
    cudaEventRecord(e, h->stream);
    h->prof->ev.push_back(e);
    h->prof->cls.push_back(cls);
}

int run_forward(gb_handle *h, const Derived *D, const double *blength, bool keepE, double *neg_lnL,
                double *fhK, double *lnf, gb_stats *stats) {
    return upload_and_run(h, D, blength, keepE, neg_lnL, fhK, lnf, stats);
}
}  // namespace gb

// ---------------------------------------------------------------- C ABI

extern "C" {

const char *gb_version(void) { return "gbcodeml 0.1 (sm_103a)"; }

const char *gb_last_error(void) { return g_err.c_str(); }

namespace {
// gb_create and gb_create_unclean: amb (nullable) is codeml's nChara[256]
// followed by CharaMap[256][64]
int create_handle(const gb_problem *prob, const unsigned char *amb, gb_handle **out) {
    if (!prob || !out) return fail(GB_ERR_ARG, "null argument");
    *out = nullptr;
    int prec = prob->precision, slices = 8;
    if (prec >= GB_PREC_FAST_NS(5) && prec <= GB_PREC_FAST_NS(8)) {
        slices = prec - GB_PREC_FAST_NS(0);
        prec = GB_PREC_FAST;
    }
    if (prec != GB_PREC_FP64 && prec != GB_PREC_FAST) return fail(GB_ERR_ARG, "unknown precision");
    // validate everything on the host before touching a device
    gb_handle *h = new gb_handle();
    h->device = -1;
    h->precision = prec;
    h->fast_slices = slices;
    int rc = build_schedule(h, prob);
    if (rc) { free_all(h); return rc; }
    bool unclean = false;
    for (size_t i = 0; i < (size_t)prob->ns * prob->npatt; i++) {
        const int c = prob->z[i];
        if (c < 61) continue;
        if (!amb) { free_all(h); return fail(GB_ERR_ARG, "z: codon id >= 61 (clean data; gb_create_unclean "
                                                         "takes ambiguity codes)"); }
        if (amb[c] < 1 || amb[c] > 61) {
            free_all(h);
            return fail(GB_ERR_ARG, "ambiguity code " + std::to_string(c) + " stands for no sense codon");
        }
        for (int q = 0; q < amb[c]; q++)
            if (amb[256 + 64 * c + q] >= 61) {
                free_all(h);
                return fail(GB_ERR_ARG, "ambiguity code " + std::to_string(c) + " maps to a codon id >= 61");
            }
        unclean = true;
    }
    if (unclean && prec != GB_PREC_FP64) {
        free_all(h);
        return fail(GB_ERR_ARG, "ambiguous codons: GB_PREC_FP64 only (the split-precision kernels take "
                                "clean data)");
    }
    h->pi.assign(prob->pi, prob->pi + 61);
    h->fpatt.assign(prob->fpatt, prob->fpatt + prob->npatt);
    for (double v : h->pi)
        if (!(v > 0)) { free_all(h); return fail(GB_ERR_ARG, "pi must be positive"); }
    for (double v : h->fpatt)
        if (!(v >= 0)) { free_all(h); return fail(GB_ERR_ARG, "fpatt must be >= 0"); }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { free_all(h); return fail(GB_ERR_NODEVICE, "no CUDA device"); }
    if (prob->device < 0 || prob->device >= ndev) { free_all(h); return fail(GB_ERR_ARG, "bad device ordinal"); }
    h->device = prob->device;

    auto bad = [&](int code) { free_all(h); return code; };
    if (cudaSetDevice(h->device) != cudaSuccess) return bad(fail(GB_ERR_CUDA, "cudaSetDevice"));
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&h->ev0) != cudaSuccess || cudaEventCreate(&h->ev1) != cudaSuccess)
        return bad(fail(GB_ERR_CUDA, "stream/event creation"));
    const size_t npad = h->npad;
    if ((rc = dalloc(&h->d_items, h->items.size())) || (rc = dalloc(&h->d_pairs, h->pairs.size())) ||
        (rc = dalloc(&h->d_label, h->nnode)) || (rc = dalloc(&h->d_scale_list, h->scale_list.size())) ||
        (rc = dalloc(&h->d_z, (size_t)h->ns * npad)) || (rc = dalloc(&h->d_fpatt, npad)) ||
        (rc = dalloc(&h->d_pi, 64)) || (rc = dalloc(&h->d_tnode, h->nnode)) || (rc = dalloc(&h->d_prm, 1)) ||
        (rc = dalloc(&h->d_Pt, h->pairs.size() * 64 * 64)) ||
        (rc = dalloc(&h->d_conP, h->precision == GB_PREC_FP64 ? (size_t)h->nslot * npad * 64 : 1)) ||
        (rc = dalloc(&h->d_scaleF, (size_t)std::max(h->nsslot, 1) * npad)) ||
        (rc = dalloc(&h->d_fbar, 4 * npad)) || (rc = dalloc(&h->d_ssum, 4 * npad)) ||
        (rc = dalloc(&h->d_fhK, 4 * npad)) || (rc = dalloc(&h->d_lnf, npad)) ||
        (rc = dalloc(&h->d_post, 4 * npad)) || (rc = dalloc(&h->d_partial, npad / 256 + 2)) ||
        (rc = dalloc(&h->d_out, 4)) || (rc = dalloc(&h->d_ticket, 1)))
        return bad(rc);
    if (cudaMallocHost((void **)&h->h_prm, sizeof(DevParams)) != cudaSuccess ||
        cudaMallocHost((void **)&h->h_tnode, sizeof(double) * h->nnode) != cudaSuccess ||
        cudaMallocHost((void **)&h->h_out, sizeof(double) * 64) != cudaSuccess)
        return bad(fail(GB_ERR_OOM, "cudaMallocHost"));
    std::vector<unsigned char> zpad((size_t)h->ns * npad, 0);
    for (int j = 0; j < h->ns; j++) std::memcpy(&zpad[j * npad], prob->z + (size_t)j * h->npatt, h->npatt);
    std::vector<double> fp(npad, 0.0), pi64(64, 0.0);
    std::copy(h->fpatt.begin(), h->fpatt.end(), fp.begin());
    std::copy(h->pi.begin(), h->pi.end(), pi64.begin());
    if (cudaMemcpy(h->d_items, h->items.data(), sizeof(Item) * h->items.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(h->d_pairs, h->pairs.data(), sizeof(PairDesc) * h->pairs.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(h->d_label, h->label.data(), sizeof(int) * h->nnode, cudaMemcpyHostToDevice) ||
        cudaMemcpy(h->d_scale_list, h->scale_list.data(), sizeof(int) * h->scale_list.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(h->d_z, zpad.data(), zpad.size(), cudaMemcpyHostToDevice) ||
        cudaMemcpy(h->d_fpatt, fp.data(), sizeof(double) * npad, cudaMemcpyHostToDevice) ||
        cudaMemcpy(h->d_pi, pi64.data(), sizeof(double) * 64, cudaMemcpyHostToDevice) ||
        cudaMemset(h->d_ticket, 0, sizeof(unsigned)) || cudaMemset(h->d_scaleF, 0, sizeof(double) * std::max(h->nsslot, 1) * npad) ||
        cudaMemset(h->d_post, 0, sizeof(double) * 4 * npad) || cudaMemset(h->d_fbar, 0, sizeof(double) * 4 * npad) ||
        cudaMemset(h->d_lnf, 0, sizeof(double) * npad) || init_fp64_kernels())
        return bad(fail(GB_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(cudaGetLastError())));
    if (unclean) {
        if ((rc = dalloc(&h->d_amb, (size_t)256 + 256 * 64))) return bad(rc);
        if (cudaMemcpy(h->d_amb, amb, 256 + 256 * 64, cudaMemcpyHostToDevice) != cudaSuccess)
            return bad(fail(GB_ERR_CUDA, "upload of the ambiguity tables"));
    }
    *out = h;
    return GB_OK;
}
}  // namespace

int gb_create(const gb_problem *prob, gb_handle **out) { return create_handle(prob, nullptr, out); }

int gb_create_unclean(const gb_problem *prob, const unsigned char *nchara, const unsigned char *charamap,
                      gb_handle **out) {
    if (!nchara || !charamap) return fail(GB_ERR_ARG, "null ambiguity tables");
    std::vector<unsigned char> amb((size_t)256 + 256 * 64);
    std::memcpy(amb.data(), nchara, 256);
    std::memcpy(amb.data() + 256, charamap, 256 * 64);
    return create_handle(prob, amb.data(), out);
}

int gb_destroy(gb_handle *h) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    free_all(h);
    return GB_OK;
}

int gb_nscale(const gb_handle *h) { return h ? h->nscale : GB_ERR_STATE; }

int gb_eval_uvr(gb_handle *h, const double *const U[3], const double *const V[3],
                const double *const Root[3], const double qfactor[2], const double freqK[4],
                const double *blength, double *neg_lnL, double *fhK, double *lnf, gb_stats *stats) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!U || !V || !Root || !qfactor || !freqK || !blength) return fail(GB_ERR_ARG, "null argument");
    Derived *D = new Derived;
    for (int i = 0; i < 3; i++) {
        if (!U[i] || !V[i] || !Root[i]) { delete D; return fail(GB_ERR_ARG, "null U/V/Root"); }
        std::memcpy(D->U[i], U[i], sizeof(double) * 61 * 61);
        std::memcpy(D->V[i], V[i], sizeof(double) * 61 * 61);
        std::memcpy(D->Root[i], Root[i], sizeof(double) * 61);
    }
    std::memcpy(D->qf, qfactor, sizeof(double) * 2);
    std::memcpy(D->freqK, freqK, sizeof(double) * 4);
    // the caller's eigen solutions: P = U diag(e) V formed as codeml's PMatUVRoot does
    D->sym = 0;
    double v = 0;
    int rc = upload_and_run(h, D, blength, false, &v, fhK, lnf, stats);
    delete D;
    if (!rc && neg_lnL) *neg_lnL = v;
    return rc;
}

namespace {
// gb_eval (model A: w1 = 1) and gb_eval_b (model B: w1 free)
int eval_impl(gb_handle *h, const gb_params *prm, double w1, bool free_w1, double *neg_lnL, gb_grad *grad,
              double *d_omega1, double *fhK, double *lnf, gb_stats *stats) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!prm || !prm->blength) return fail(GB_ERR_ARG, "null argument");
    double t0 = now_ms();
    Derived *D = new Derived;
    ModelParams m{prm->kappa, prm->omega0, prm->omega2, prm->p0, prm->p1};
    m.w1 = w1;
    m.free_w1 = free_w1;
    int rc = derive(h->pi.data(), m, grad != nullptr, D);
    if (rc) { delete D; return fail(rc, "model parameters out of range"); }
    double v = 0;
    if (h->precision == GB_PREC_FAST) {
        rc = fast_eval(h, D, prm->blength, &v, grad, fhK, lnf, stats);
    } else {
        // checkpointed adjoint: the forward keeps no edge messages
        rc = upload_and_run(h, D, prm->blength, grad != nullptr && !h->tune.checkpoint, &v, fhK, lnf, stats);
        if (!rc && grad) rc = adjoint_run(h, D, m, prm->blength, grad, stats);
    }
    delete D;
    if (rc) return rc;
    if (neg_lnL) *neg_lnL = v;
    if (grad && d_omega1) *d_omega1 = h->adj ? h->adj->d_omega1 : 0.0;
    if (stats) stats->ms_host = now_ms() - t0;
    return GB_OK;
}
}  // namespace

int gb_eval(gb_handle *h, const gb_params *prm, double *neg_lnL, gb_grad *grad, double *fhK,
            double *lnf, gb_stats *stats) {
    return eval_impl(h, prm, 1.0, false, neg_lnL, grad, nullptr, fhK, lnf, stats);
}

int gb_eval_b(gb_handle *h, const gb_params *prm, double omega1, double *neg_lnL, gb_grad *grad,
              double *d_omega1, double *fhK, double *lnf, gb_stats *stats) {
    return eval_impl(h, prm, omega1, true, neg_lnL, grad, d_omega1, fhK, lnf, stats);
}

int gb_neb(gb_handle *h, const gb_params *prm, double *post, double *neg_lnL) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    if (!prm || !prm->blength || !post) return fail(GB_ERR_ARG, "null argument");
    if (h->precision != GB_PREC_FP64) return fail(GB_ERR_STATE, "gb_neb needs a GB_PREC_FP64 handle");
    Derived *D = new Derived;
    ModelParams m{prm->kappa, prm->omega0, prm->omega2, prm->p0, prm->p1};
    int rc = derive(h->pi.data(), m, false, D);
    if (rc) { delete D; return fail(rc, "model parameters out of range"); }
    double v = 0;
    rc = upload_and_run(h, D, prm->blength, false, &v, nullptr, nullptr, nullptr);
    delete D;
    if (rc) return rc;
    // the mixture kernel's class posteriors of the evaluation just run
    CK(cudaMemcpy2D(post, sizeof(double) * h->npatt, h->d_post, sizeof(double) * h->npad,
                    sizeof(double) * h->npatt, 4, cudaMemcpyDeviceToHost));
    if (neg_lnL) *neg_lnL = v;
    return GB_OK;
}

int gb_dfun_x(gb_handle *h, const int *bnode, int lastround, const double *x, int n, double *f,
              double *dx) {
    if (!h) return fail(GB_ERR_STATE, "null handle");
    const int nb = h->nnode - 1;
    // model A: x ends kappa, p0', p1', w0, w2; model B (n = nb + 6): ..., w0, w1, w2
    if (!bnode || !x || !f || !dx || (n != nb + 5 && n != nb + 6)) return fail(GB_ERR_ARG, "gb_dfun_x: bad arguments");
    const bool model_b = n == nb + 6;
    const int iw2 = model_b ? nb + 5 : nb + 4;
    std::vector<double> bl(h->nnode, 0.0), dbl(h->nnode, 0.0);
    for (int ib = 0; ib < nb; ib++) {
        if (bnode[ib] < 0 || bnode[ib] >= h->nnode || bnode[ib] == h->root) return fail(GB_ERR_ARG, "bnode");
        bl[bnode[ib]] = x[ib];
    }
    gb_params p{bl.data(), x[nb], x[nb + 3], x[iw2], 0, 0};
    double e1 = 0, e2 = 0;
    if (!lastround) {   // codeml's f_and_x: p_i = e^{x_i} / (1 + e^{x_1} + e^{x_2})
        e1 = std::exp(x[nb + 1]);
        e2 = std::exp(x[nb + 2]);
        double tot = 1 + e1 + e2;
        p.p0 = e1 / tot;
        p.p1 = e2 / tot;
    } else {
        p.p0 = x[nb + 1];
        p.p1 = x[nb + 2];
    }
    gb_grad g{dbl.data(), 0, 0, 0, 0, 0};
    double dw1 = 0;
    int rc = model_b ? gb_eval_b(h, &p, x[nb + 4], f, &g, &dw1, nullptr, nullptr, nullptr)
                     : gb_eval(h, &p, f, &g, nullptr, nullptr, nullptr);
    if (rc) return rc;
    for (int ib = 0; ib < nb; ib++) dx[ib] = dbl[bnode[ib]];
    dx[nb] = g.d_kappa;
    if (!lastround) {
        dx[nb + 1] = g.d_p0 * p.p0 * (1 - p.p0) - g.d_p1 * p.p0 * p.p1;
        dx[nb + 2] = -g.d_p0 * p.p0 * p.p1 + g.d_p1 * p.p1 * (1 - p.p1);
    } else {
        dx[nb + 1] = g.d_p0;
        dx[nb + 2] = g.d_p1;
    }
    dx[nb + 3] = g.d_omega0;
    if (model_b) dx[nb + 4] = dw1;
    dx[iw2] = g.d_omega2;
    return GB_OK;
}

int gb_replay(gb_handle *h, int iters, int with_grad, double *ms) {
    if (!h || !ms || iters < 1) return fail(GB_ERR_ARG, "gb_replay: bad arguments");
    if (h->precision == GB_PREC_FAST) return fast_replay(h, iters, with_grad, ms);
    cudaGraphExec_t g = h->graph[(with_grad && !h->tune.checkpoint) ? 1 : 0];
    if (!g || (with_grad && !adjoint_ready(h))) return fail(GB_ERR_STATE, "gb_replay: evaluate first");
    CK(cudaSetDevice(h->device));
    CK(cudaEventRecord(h->ev0, h->stream));
    for (int i = 0; i < iters; i++) {
        CK(cudaGraphLaunch(g, h->stream));
        if (with_grad) {
            int rc = adjoint_launch_graph(h);
            if (rc) return rc;
        }
    }
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    float t = 0;
    CK(cudaEventElapsedTime(&t, h->ev0, h->ev1));
    *ms = t;
    return GB_OK;
}

int gb_profile(gb_handle *h, int iters, int with_grad, double *ms, int *launches) {
    if (!h || !ms || !launches || iters < 1) return fail(GB_ERR_ARG, "gb_profile: bad arguments");
    if (h->precision == GB_PREC_FAST) return fast_profile(h, iters, with_grad, ms, launches);
    if (!h->graph[(with_grad && !h->tune.checkpoint) ? 1 : 0] || (with_grad && !adjoint_ready(h)))
        return fail(GB_ERR_STATE, "gb_profile: evaluate first");
    CK(cudaSetDevice(h->device));
    ProfRec rec;
    h->prof = &rec;
    prof_mark(h, -1);
    for (int i = 0; i < iters; i++) {
        record_forward(h, with_grad != 0 && !h->tune.checkpoint);
        if (with_grad) adjoint_record(h);
    }
    h->prof = nullptr;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    for (int k = 0; k < GB_NKCLASS; k++) { ms[k] = 0; launches[k] = 0; }
    for (size_t i = 1; i < rec.ev.size(); i++) {
        float t = 0;
        cudaEventElapsedTime(&t, rec.ev[i - 1], rec.ev[i]);
        int c = rec.cls[i];
        if (c >= 0 && c < GB_NKCLASS) { ms[c] += t; launches[c]++; }
    }
    for (auto ev : rec.ev) cudaEventDestroy(ev);
    if (e != cudaSuccess) return cuda_fail(e, "gb_profile");
    return GB_OK;
}

int gb_tune(gb_handle *h, int knob, int value) {
    if (!h) return fail(GB_ERR_ARG, "gb_tune: null handle");
    if (h->fast || h->adj) return fail(GB_ERR_STATE, "gb_tune: handle already evaluated");
    switch (knob) {
        case GB_TUNE_MMA:
        case GB_TUNE_PERSIST:
            if (value != 0 && value != 1) return fail(GB_ERR_ARG, "gb_tune: value must be 0 or 1");
            (knob == GB_TUNE_MMA ? h->tune.mma : h->tune.persist) = value;
            return GB_OK;
        case GB_TUNE_GCHUNK:
            if (value < 64 || value > 8192 || value % 64) return fail(GB_ERR_ARG, "gb_tune: chunk must be a multiple of 64 in [64, 8192]");
            h->tune.gchunk = value;
            return GB_OK;
        case GB_TUNE_ORDER:
            if (value < 0 || value > 2) return fail(GB_ERR_ARG, "gb_tune: order must be 0, 1 or 2");
            h->tune.order = value;
            return GB_OK;
        case GB_TUNE_GRID:
            if (value < 0) return fail(GB_ERR_ARG, "gb_tune: grid must be >= 0");
            h->tune.grid = value;
            return GB_OK;
        case GB_TUNE_CHECKPOINT:
            if (value != 0 && value != 1) return fail(GB_ERR_ARG, "gb_tune: value must be 0 or 1");
            if (value && h->precision != GB_PREC_FP64)
                return fail(GB_ERR_ARG, "gb_tune: the checkpointed adjoint is on the FP64 path");
            h->tune.checkpoint = value;
            return GB_OK;
        default:
            return fail(GB_ERR_ARG, "gb_tune: unknown knob");
    }
}

int gb_task_trace(gb_handle *h, int kernel, unsigned long long *out, int cap) {
    if (!h || cap < 0) return fail(GB_ERR_ARG, "gb_task_trace: bad arguments");
    return fast_task_trace(h, kernel, out, cap);
}

int gb_fault_inject(gb_handle *h, int wait_ms, int withhold) {
    if (!h) return fail(GB_ERR_ARG, "gb_fault_inject: null handle");
    return fast_fault_inject(h, wait_ms, withhold);
}

int gb_model_setup(const double *pi, double kappa, double omega0, double omega2, double p0, double p1,
                   double *U, double *V, double *Root, double *qf, double *freqK) {
    if (!pi) return fail(GB_ERR_ARG, "null pi");
    Derived *D = new Derived;
    int rc = derive(pi, ModelParams{kappa, omega0, omega2, p0, p1}, false, D);
    if (!rc) {
        for (int i = 0; i < 3; i++) {
            if (U) std::memcpy(U + i * 61 * 61, D->U[i], sizeof(double) * 61 * 61);
            if (V) std::memcpy(V + i * 61 * 61, D->V[i], sizeof(double) * 61 * 61);
            if (Root) std::memcpy(Root + i * 61, D->Root[i], sizeof(double) * 61);
        }
        if (qf) std::memcpy(qf, D->qf, sizeof(double) * 2);
        if (freqK) std::memcpy(freqK, D->freqK, sizeof(double) * 4);
    }
    delete D;
    return rc ? fail(rc, "model parameters out of range") : GB_OK;
}

}  // extern "C"

