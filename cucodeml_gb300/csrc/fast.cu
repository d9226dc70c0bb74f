// Host side of the split-precision path (GB_PREC_FAST): buffers, CUDA graphs
// and launches; the kernels are in k_fast.cu (forward).
#include <cuda_runtime.h>

#include <cstring>

#include "fast_internal.h"
#include "handle.h"

namespace gb {

struct FastState {
    int ns = 8;                  // digit planes per operand
    float2 *Pdf = nullptr, *conP = nullptr, *E = nullptr;
    __nv_bfloat16 *Bf = nullptr, *Bb = nullptr;
    int *expo = nullptr, *expo_root = nullptr;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_kernels = 0;
};

void fast_free(FastState *f) {
    if (!f) return;
    for (auto &g : f->graph)
        if (g) cudaGraphExecDestroy(g);
    void *p[] = {f->Pdf, f->conP, f->E, f->Bf, f->Bb, f->expo, f->expo_root};
    for (void *q : p)
        if (q) cudaFree(q);
    delete f;
}

namespace {

int fast_init(gb_handle *h) {
    FastState *f = new FastState();
    h->fast = f;
    f->ns = h->fast_slices;
    const size_t npad = h->npad, np = h->pairs.size();
    int rc;
    if ((rc = dalloc(&f->Pdf, np * 4096)) || (rc = dalloc(&f->Bf, np * f->ns * 4096)) ||
        (rc = dalloc(&f->Bb, np * f->ns * 4096)) || (rc = dalloc(&f->conP, (size_t)h->nslot * npad * 64)) ||
        (rc = dalloc(&f->expo, (size_t)h->nslot * npad)) || (rc = dalloc(&f->expo_root, 4 * npad)))
        return rc;
    CK(cudaMemset(f->expo, 0, sizeof(int) * h->nslot * npad));
    CK(init_fast_kernels(f->ns));
    return 0;
}

FastFwdArgs fwd_args(gb_handle *h, bool keepE) {
    FastState *f = h->fast;
    FastFwdArgs a;
    a.items = h->d_items;
    a.npad = h->npad;
    a.z = h->d_z;
    a.Pt64 = h->d_Pt;
    a.Pdf = f->Pdf;
    a.Bf = f->Bf;
    a.Bb = f->Bb;
    a.conP = f->conP;
    a.expo = f->expo;
    a.E = keepE ? f->E : nullptr;
    a.pi = h->d_pi;
    a.fbar = h->d_fbar;
    a.ssum = h->d_ssum;
    a.fhK = h->d_fhK;
    a.expo_root = f->expo_root;
    return a;
}

int record_forward_fast(gb_handle *h, bool keepE) {
    FastState *f = h->fast;
    int nk = 0;
    launch_pmat_fp64(h->d_pairs, (int)h->pairs.size(), h->d_label, h->d_tnode, h->d_prm, h->d_Pt, h->stream);
    prof_mark(h, GB_K_PMAT);
    nk++;
    FastFwdArgs a = fwd_args(h, keepE);
    launch_pslice(a, f->ns, (int)h->pairs.size(), h->stream);
    prof_mark(h, GB_K_PMAT);
    nk++;
    const int ntile = h->npad / FAST_MT;
    const int H = (int)h->level_off.size() - 1;
    for (int L = 0; L < H; L++) {
        const int n = h->level_off[L + 1] - h->level_off[L];
        if (!n) continue;
        FastFwdArgs al = a;
        al.items = h->d_items + h->level_off[L];
        launch_prune_fast(al, f->ns, n, ntile, h->stream);
        prof_mark(h, GB_K_PRUNE);
        nk++;
    }
    // every node is renormalised, so fhK is always in log form
    launch_mix(h->d_fhK, h->d_fpatt, h->d_prm, h->npatt, h->npad, 1, h->d_lnf, h->d_post, h->d_partial,
               h->d_ticket, h->d_out, h->stream);
    prof_mark(h, GB_K_MIX);
    nk++;
    return nk;
}

int ensure_fast_graph(gb_handle *h, bool keepE) {
    FastState *f = h->fast;
    cudaGraphExec_t &ge = f->graph[keepE ? 1 : 0];
    if (ge) return 0;
    if (keepE && !f->E) {
        int rc = dalloc(&f->E, (size_t)h->nslot * MAXC * h->npad * 64);
        if (rc) return rc;
    }
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    f->graph_kernels = record_forward_fast(h, keepE);
    CK(cudaStreamEndCapture(h->stream, &g));
    cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (fast)");
    return 0;
}

}  // namespace

int fast_eval(gb_handle *h, const Derived *D, const double *blength, double *neg_lnL, gb_grad *grad,
              double *fhK, double *lnf, gb_stats *stats) {
    if (grad) return fail(GB_ERR_STATE, "GB_PREC_FAST: the gradient is not available in this build");
    CK(cudaSetDevice(h->device));
    if (!h->fast) {
        int rc = fast_init(h);
        if (rc) return rc;
    }
    FastState *f = h->fast;
    double t0 = now_ms();
    for (int i = 0; i < 3; i++) {
        std::memcpy(h->h_prm->U[i], D->U[i], sizeof(double) * 61 * 61);
        std::memcpy(h->h_prm->V[i], D->V[i], sizeof(double) * 61 * 61);
        std::memcpy(h->h_prm->Root[i], D->Root[i], sizeof(double) * 61);
    }
    std::memcpy(h->h_prm->qf, D->qf, sizeof(double) * 2);
    std::memcpy(h->h_prm->freqK, D->freqK, sizeof(double) * 4);
    for (int n = 0; n < h->nnode; n++) {
        double t = n == h->root ? 0.0 : blength[n];
        if (!(t >= 0.0)) return fail(GB_ERR_PARAM, "negative or non-finite branch length");
        h->h_tnode[n] = t;
    }
    const bool keepE = false;
    int rc = ensure_fast_graph(h, keepE);
    if (rc) return rc;
    CK(cudaEventRecord(h->ev0, h->stream));
    CK(cudaMemcpyAsync(h->d_prm, h->h_prm, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_tnode, h->h_tnode, sizeof(double) * h->nnode, cudaMemcpyHostToDevice, h->stream));
    CK(cudaGraphLaunch(f->graph[keepE ? 1 : 0], h->stream));
    CK(cudaMemcpyAsync(h->h_out, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    if (fhK)
        CK(cudaMemcpy2DAsync(fhK, sizeof(double) * h->npatt, h->d_fhK, sizeof(double) * h->npad,
                             sizeof(double) * h->npatt, 4, cudaMemcpyDeviceToHost, h->stream));
    if (lnf) CK(cudaMemcpyAsync(lnf, h->d_lnf, sizeof(double) * h->npatt, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    *neg_lnL = h->h_out[0];
    h->kernels_last = f->graph_kernels;
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        stats->ms_device = ms;
        stats->ms_host = now_ms() - t0;
        stats->kernels = f->graph_kernels;
        stats->nscale = h->nscale;
        stats->h2d_bytes = sizeof(DevParams) + sizeof(double) * h->nnode;
        stats->d2h_bytes = sizeof(double) * (1 + (fhK ? 4 * h->npatt : 0) + (lnf ? h->npatt : 0));
    }
    return 0;
}

int fast_replay(gb_handle *h, int iters, int with_grad, double *ms) {
    if (with_grad) return fail(GB_ERR_STATE, "GB_PREC_FAST: the gradient is not available in this build");
    if (!h->fast || !h->fast->graph[0]) return fail(GB_ERR_STATE, "gb_replay: evaluate first");
    CK(cudaSetDevice(h->device));
    CK(cudaEventRecord(h->ev0, h->stream));
    for (int i = 0; i < iters; i++) CK(cudaGraphLaunch(h->fast->graph[0], h->stream));
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    float t = 0;
    CK(cudaEventElapsedTime(&t, h->ev0, h->ev1));
    *ms = t;
    return 0;
}

int fast_profile(gb_handle *h, int iters, int with_grad, double *ms, int *launches) {
    if (with_grad) return fail(GB_ERR_STATE, "GB_PREC_FAST: the gradient is not available in this build");
    if (!h->fast || !h->fast->graph[0]) return fail(GB_ERR_STATE, "gb_profile: evaluate first");
    CK(cudaSetDevice(h->device));
    ProfRec rec;
    h->prof = &rec;
    prof_mark(h, -1);
    for (int i = 0; i < iters; i++) record_forward_fast(h, false);
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
    if (e != cudaSuccess) return cuda_fail(e, "gb_profile (fast)");
    return 0;
}

}  // namespace gb
