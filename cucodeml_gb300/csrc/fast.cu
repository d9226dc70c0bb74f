// Host side of the split-precision path (GB_PREC_FAST): buffers, CUDA graphs
// and launches.  Kernels: k_umma.cu (tcgen05 contractions, the default),
// k_fast.cu / k_fast_bwd.cu (mma.sync contractions, P digit planes, dlnL/dP).
// GBCODEML_MMA=sync in the environment selects the mma.sync contraction
// kernels for the forward and adjoint levels.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>

#include "adjoint_internal.h"
#include "fast_internal.h"
#include "handle.h"

namespace gb {

struct FastState {
    int ns = 8;                  // digit planes per operand
    float2 *Pdf = nullptr, *conP = nullptr, *E = nullptr;
    __nv_bfloat16 *Bf = nullptr, *Bb = nullptr;
    int *expo = nullptr, *expo_root = nullptr;
    int *ebexp = nullptr, *aexp = nullptr;     // adjoint exponents
    int *err = nullptr, *h_err = nullptr;      // bounded-wait failure flag (device, pinned host)
    bool umma = true;                          // tcgen05 contractions (else mma.sync)
    int nsb = 7;                               // digit planes in the adjoint contractions
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    cudaGraphExec_t bwd_graph = nullptr;
    int graph_kernels = 0, bwd_kernels = 0;
};

void fast_free(FastState *f) {
    if (!f) return;
    for (auto &g : f->graph)
        if (g) cudaGraphExecDestroy(g);
    if (f->bwd_graph) cudaGraphExecDestroy(f->bwd_graph);
    if (f->h_err) cudaFreeHost(f->h_err);
    void *p[] = {f->Pdf, f->conP, f->E, f->Bf, f->Bb, f->expo, f->expo_root, f->ebexp, f->aexp, f->err};
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
    const char *mode = std::getenv("GBCODEML_MMA");
    const char *nb = std::getenv("GBCODEML_ADJ_PLANES");
    f->nsb = nb ? std::atoi(nb) : 7;
    if (f->nsb < 4 || f->nsb > f->ns) f->nsb = f->ns < 7 ? f->ns : 7;
    f->umma = !(mode && std::strcmp(mode, "sync") == 0) && f->ns >= 6;
    if ((rc = dalloc(&f->err, 1))) return rc;
    CK(cudaMemset(f->err, 0, sizeof(int)));
    CK(cudaMallocHost((void **)&f->h_err, sizeof(int)));
    CK(init_fast_kernels(f->ns));
    if (f->umma) {
        CK(init_umma_kernels(f->ns));
        CK(init_umma_kernels(f->nsb));
    }
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
    a.err = f->err;
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
        if (f->umma) launch_prune_umma(al, f->ns, n, ntile, h->stream);
        else launch_prune_fast(al, f->ns, n, ntile, h->stream);
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

FastBwdArgs bwd_args(gb_handle *h) {
    FastState *f = h->fast;
    AdjointState *ad = h->adj;
    FastBwdArgs b;
    b.bitems = ad->d_bitems;
    b.npad = h->npad;
    b.npatt = h->npatt;
    b.nchunk = ad->nchunk;
    b.E = f->E;
    b.conP = f->conP;
    b.expo = f->expo;
    b.expo_root = f->expo_root;
    b.Bb = f->Bb;
    // the FP64 adjoint's message buffers hold 8 bytes per element: reused as double-float
    b.Ebar = reinterpret_cast<float2 *>(ad->d_Ebar);
    b.ebexp = f->ebexp;
    b.Abar = reinterpret_cast<float2 *>(ad->d_Abar);
    b.aexp = f->aexp;
    b.fpatt = h->d_fpatt;
    b.post = h->d_post;
    b.fbar = h->d_fbar;
    b.pi = h->d_pi;
    b.contrib = ad->d_contrib;
    b.coff = ad->d_coff;
    b.z = h->d_z;
    b.Gpart = ad->d_Gpart;
    b.err = f->err;
    b.nsP = f->ns;
    b.gchunk = GCHUNK;
    return b;
}

int record_backward_fast(gb_handle *h) {
    FastState *f = h->fast;
    AdjointState *ad = h->adj;
    int nk = 0;
    launch_dmat(h);
    prof_mark(h, GB_K_OTHER);
    nk++;
    FastBwdArgs b = bwd_args(h);
    const int ntile = h->npad / FAST_MT;
    for (size_t L = 0; L + 1 < ad->blevel_off.size(); L++) {
        const int n = ad->blevel_off[L + 1] - ad->blevel_off[L];
        if (!n) continue;
        FastBwdArgs bl = b;
        bl.bitems = ad->d_bitems + ad->blevel_off[L];
        if (f->umma) launch_bwd_umma(bl, f->nsb, n, ntile, h->stream);
        else launch_bwd_fast(bl, f->ns, n, ntile, h->stream);
        prof_mark(h, GB_K_BWD);
        nk++;
    }
    if (f->umma) launch_gradP_umma(b, f->nsb, (int)h->pairs.size(), h->stream);
    else launch_gradP_fast(b, f->ns, (int)h->pairs.size(), h->stream);
    prof_mark(h, GB_K_GRADP);
    nk++;
    launch_gradH(h);
    prof_mark(h, GB_K_GRADH);
    nk++;
    launch_freq(h, 1);
    prof_mark(h, GB_K_OTHER);
    nk++;
    return nk;
}

int ensure_bwd_graph(gb_handle *h) {
    FastState *f = h->fast;
    if (f->bwd_graph) return 0;
    int rc = adjoint_init(h);
    if (rc) return rc;
    if (!f->ebexp) {
        if ((rc = dalloc(&f->ebexp, (size_t)h->nslot * MAXC * h->npad)) ||
            (rc = dalloc(&f->aexp, (size_t)h->nslot * h->npad)))
            return rc;
        CK(cudaMemset(f->aexp, 0, sizeof(int) * h->nslot * h->npad));
    }
    CK(init_fast_bwd_kernels(f->ns));
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    f->bwd_kernels = record_backward_fast(h);
    CK(cudaStreamEndCapture(h->stream, &g));
    cudaError_t e = cudaGraphInstantiate(&f->bwd_graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (fast adjoint)");
    return 0;
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

int fast_prepare(gb_handle *h, bool grad) {
    CK(cudaSetDevice(h->device));
    if (!h->fast) {
        int rc = fast_init(h);
        if (rc) return rc;
    }
    int rc = ensure_fast_graph(h, grad);
    if (!rc && grad) rc = ensure_bwd_graph(h);
    return rc;
}

int fast_record_eval(gb_handle *h, bool grad) {
    FastState *f = h->fast;
    CK(cudaMemcpyAsync(h->d_prm, h->h_prm, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_tnode, h->h_tnode, sizeof(double) * h->nnode, cudaMemcpyHostToDevice, h->stream));
    if (grad) CK(cudaMemcpyAsync(h->adj->d_gp, h->adj->h_gp, sizeof(GradParams), cudaMemcpyHostToDevice, h->stream));
    int nk = record_forward_fast(h, grad);
    if (grad) {
        nk += record_backward_fast(h);
        int rc = adjoint_fetch(h);
        if (rc) return -rc;
    }
    CK(cudaMemcpyAsync(h->h_out, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(f->h_err, f->err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    return nk;
}

int fast_check_error(gb_handle *h) {
    FastState *f = h->fast;
    if (f && *f->h_err) {
        cudaMemset(f->err, 0, sizeof(int));
        *f->h_err = 0;
        return fail(GB_ERR_TIMEOUT, "a tensor-core completion wait gave up (bounded mbarrier wait)");
    }
    return 0;
}

int fast_eval(gb_handle *h, const Derived *D, const double *blength, double *neg_lnL, gb_grad *grad,
              double *fhK, double *lnf, gb_stats *stats) {
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
    const bool keepE = grad != nullptr;
    int rc = ensure_fast_graph(h, keepE);
    if (rc) return rc;
    if (grad) {
        rc = ensure_bwd_graph(h);
        if (rc) return rc;
        std::memcpy(h->adj->h_gp->dQk, D->dQk, sizeof(D->dQk));
        std::memcpy(h->adj->h_gp->dQw, D->dQw, sizeof(D->dQw));
    }
    CK(cudaEventRecord(h->ev0, h->stream));
    CK(cudaMemcpyAsync(h->d_prm, h->h_prm, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_tnode, h->h_tnode, sizeof(double) * h->nnode, cudaMemcpyHostToDevice, h->stream));
    if (grad) CK(cudaMemcpyAsync(h->adj->d_gp, h->adj->h_gp, sizeof(GradParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaGraphLaunch(f->graph[keepE ? 1 : 0], h->stream));
    if (grad) {
        CK(cudaGraphLaunch(f->bwd_graph, h->stream));
        rc = adjoint_fetch(h);
        if (rc) return rc;
    }
    CK(cudaMemcpyAsync(h->h_out, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(f->h_err, f->err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    if (fhK)
        CK(cudaMemcpy2DAsync(fhK, sizeof(double) * h->npatt, h->d_fhK, sizeof(double) * h->npad,
                             sizeof(double) * h->npatt, 4, cudaMemcpyDeviceToHost, h->stream));
    if (lnf) CK(cudaMemcpyAsync(lnf, h->d_lnf, sizeof(double) * h->npatt, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    if (*f->h_err) {
        cudaMemset(f->err, 0, sizeof(int));
        return fail(GB_ERR_TIMEOUT, "a tensor-core completion wait gave up (bounded mbarrier wait)");
    }
    *neg_lnL = h->h_out[0];
    h->kernels_last = f->graph_kernels + (grad ? f->bwd_kernels : 0);
    if (grad) adjoint_chain(h, D, blength, grad);
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        stats->ms_device = ms;
        stats->ms_host = now_ms() - t0;
        stats->kernels = h->kernels_last;
        stats->nscale = h->nscale;
        stats->h2d_bytes = sizeof(DevParams) + sizeof(double) * h->nnode + (grad ? sizeof(GradParams) : 0);
        stats->d2h_bytes = sizeof(double) * (1 + (fhK ? 4 * h->npatt : 0) + (lnf ? h->npatt : 0)) +
                           (grad ? sizeof(double) * (h->pairs.size() * 3 + h->adj->nfreq_blocks * 4) : 0);
    }
    return 0;
}

int fast_replay(gb_handle *h, int iters, int with_grad, double *ms) {
    FastState *f = h->fast;
    if (!f || !f->graph[with_grad ? 1 : 0] || (with_grad && !f->bwd_graph))
        return fail(GB_ERR_STATE, "gb_replay: evaluate first");
    CK(cudaSetDevice(h->device));
    CK(cudaEventRecord(h->ev0, h->stream));
    for (int i = 0; i < iters; i++) {
        CK(cudaGraphLaunch(f->graph[with_grad ? 1 : 0], h->stream));
        if (with_grad) CK(cudaGraphLaunch(f->bwd_graph, h->stream));
    }
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    float t = 0;
    CK(cudaEventElapsedTime(&t, h->ev0, h->ev1));
    *ms = t;
    return 0;
}

int fast_profile(gb_handle *h, int iters, int with_grad, double *ms, int *launches) {
    FastState *f = h->fast;
    if (!f || !f->graph[with_grad ? 1 : 0] || (with_grad && !f->bwd_graph))
        return fail(GB_ERR_STATE, "gb_profile: evaluate first");
    CK(cudaSetDevice(h->device));
    ProfRec rec;
    h->prof = &rec;
    prof_mark(h, -1);
    for (int i = 0; i < iters; i++) {
        record_forward_fast(h, with_grad != 0);
        if (with_grad) record_backward_fast(h);
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
    if (e != cudaSuccess) return cuda_fail(e, "gb_profile (fast)");
    return 0;
}

}  // namespace gb
