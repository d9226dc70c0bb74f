// Host side of the split-precision path (GB_PREC_FAST): buffers, CUDA graphs
// and launches.  Kernels: k_umma.cu (tcgen05 contractions, the default),
// k_fast.cu / k_fast_bwd.cu (mma.sync contractions, P digit planes, dlnL/dP).
// GBCODEML_MMA=sync in the environment selects the mma.sync contraction
// kernels for the forward and adjoint levels; GBCODEML_PERSIST=0 selects one
// tcgen05 launch per tree level instead of the persistent task-list kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "adjoint_internal.h"
#include "fast_internal.h"
#include "handle.h"
#include "batch_internal.h"

namespace gb {

struct FastState {
    int ns = 8;                  // digit planes per operand
    float2 *Pdf = nullptr, *conP = nullptr, *E = nullptr;
    __nv_bfloat16 *Bf = nullptr, *Bb = nullptr;
    int *expo = nullptr, *expo_root = nullptr;
    int *ebexp = nullptr, *aexp = nullptr;     // adjoint exponents
    float2 *groot = nullptr;                   // [4][npad] adjoint root seed (written by the mixture)
    float2 *pidf = nullptr;                    // [64] codon frequencies as double-float (zero padded)
    int *err = nullptr, *h_err = nullptr;      // bounded-wait failure flag (device, pinned host)
    bool umma = true;                          // tcgen05 contractions (else mma.sync)
    bool persist = true;                       // persistent task-list kernels (tcgen05 only)
    int nsb = 7;                               // digit planes in the adjoint contractions
    unsigned *ready_f = nullptr, *ready_b = nullptr;   // [nslot][ntile] forward / adjoint ready flags
    PersistPlan plan;                          // this handle's own persistent launches
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
    persist_free(&f->plan);
    void *p[] = {f->Pdf, f->conP, f->E, f->Bf, f->Bb, f->expo, f->expo_root, f->ebexp, f->aexp, f->err,
                 f->ready_f, f->ready_b, f->groot, f->pidf};
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
    const char *ps = std::getenv("GBCODEML_PERSIST");
    f->persist = !(ps && std::strcmp(ps, "0") == 0);
    if (h->tune.mma >= 0) f->umma = h->tune.mma != 0 && f->ns >= 6;
    if (h->tune.persist >= 0) f->persist = h->tune.persist != 0;
    f->persist = f->persist && f->umma;
    const size_t nflag = (size_t)h->nslot * (npad / FAST_MT);
    if ((rc = dalloc(&f->ready_f, nflag)) || (rc = dalloc(&f->ready_b, nflag))) return rc;
    CK(cudaMemset(f->ready_f, 0, sizeof(unsigned) * std::max<size_t>(nflag, 1)));
    CK(cudaMemset(f->ready_b, 0, sizeof(unsigned) * std::max<size_t>(nflag, 1)));
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
    a.ready = f->ready_f;
    a.ntile = h->npad / FAST_MT;
    return a;
}

int rec_levels_fwd(gb_handle *h, bool keepE) {
    FastState *f = h->fast;
    FastFwdArgs a = fwd_args(h, keepE);
    const int ntile = h->npad / FAST_MT;
    const int H = (int)h->level_off.size() - 1;
    int nk = 0;
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
    return nk;
}

int record_forward_fast(gb_handle *h, bool keepE) {
    FastState *f = h->fast;
    int nk = 0;
    if (f->persist) {
        launch_bump(f->plan.ctl, h->stream);
        prof_mark(h, GB_K_OTHER);
        nk++;
    }
    nk += fast_rec_pmat(h);
    if (f->persist) nk += persist_record_fwd(&f->plan, keepE, f->ns, h->stream, h);
    else nk += rec_levels_fwd(h, keepE);
    nk += fast_rec_mix(h);
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
    b.groot = f->groot;
    b.pidf = f->pidf;
    b.contrib = ad->d_contrib;
    b.coff = ad->d_coff;
    b.z = h->d_z;
    // the FP64 partials buffer holds 8 bytes per element: reused as double-float
    b.Gpart = reinterpret_cast<float2 *>(ad->d_Gpart);
    b.err = f->err;
    b.nsP = f->ns;
    b.gchunk = ad->gchunk;
    b.ready = f->ready_b;
    b.ntile = h->npad / FAST_MT;
    b.Pdf = f->Pdf;
    return b;
}

int rec_levels_bwd(gb_handle *h) {
    FastState *f = h->fast;
    AdjointState *ad = h->adj;
    int nk = 0;
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
    return nk;
}

int record_backward_fast(gb_handle *h) {
    FastState *f = h->fast;
    int nk = fast_rec_dmat(h);
    if (f->persist) nk += persist_record_bwd(&f->plan, f->nsb, h->stream, h);
    else nk += rec_levels_bwd(h);
    nk += fast_rec_tail(h);
    return nk;
}

// buffers of an evaluation with (grad) or without the adjoint; no graph
int fast_alloc(gb_handle *h, bool grad) {
    if (!h->fast) {
        int rc = fast_init(h);
        if (rc) return rc;
    }
    FastState *f = h->fast;
    if (!grad) return 0;
    int rc;
    if (!f->E && (rc = dalloc(&f->E, (size_t)h->nslot * MAXC * h->npad * 64))) return rc;
    if ((rc = adjoint_init(h))) return rc;
    if (!f->ebexp) {
        if ((rc = dalloc(&f->ebexp, (size_t)h->nslot * MAXC * h->npad)) ||
            (rc = dalloc(&f->aexp, (size_t)h->nslot * h->npad)) || (rc = dalloc(&f->groot, 4 * h->npad)) ||
            (rc = dalloc(&f->pidf, 64)))
            return rc;
        CK(cudaMemset(f->aexp, 0, sizeof(int) * h->nslot * h->npad));
        CK(cudaMemset(f->groot, 0, sizeof(float2) * 4 * h->npad));   // padded patterns stay 0
        std::vector<float2> pd(64, make_float2(0.f, 0.f));
        for (int j = 0; j < 61; j++) {
            const float hi = (float)h->pi[j];
            pd[j] = make_float2(hi, (float)(h->pi[j] - (double)hi));
        }
        CK(cudaMemcpy(f->pidf, pd.data(), sizeof(float2) * 64, cudaMemcpyHostToDevice));
        CK(init_fast_bwd_kernels(f->ns));
    }
    return 0;
}

int ensure_bwd_graph(gb_handle *h) {
    FastState *f = h->fast;
    if (f->bwd_graph) return 0;
    int rc = fast_alloc(h, true);
    if (rc) return rc;
    if (f->persist) {
        gb_handle *one[1] = {h};
        if ((rc = persist_build(&f->plan, one, 1, true, h->tune))) return rc;
    }
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
    int rc = fast_alloc(h, keepE);
    if (rc) return rc;
    if (f->persist) {
        gb_handle *one[1] = {h};
        if ((rc = persist_build(&f->plan, one, 1, keepE, h->tune))) return rc;
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

// ---------------------------------------------------------------- persistent plans

void persist_free(PersistPlan *pp) {
    void *p[] = {pp->ctl,     pp->d_fargs[0], pp->d_fargs[1], pp->d_bargs, pp->d_ftask,
                 pp->d_btask, pp->d_gtask,    pp->trace[0],   pp->trace[1], pp->trace[2]};
    for (void *q : p)
        if (q) cudaFree(q);
    *pp = PersistPlan();
}

int persist_build(PersistPlan *pp, gb_handle *const *hs, int n, bool bwd, const Tuning &tune) {
    int rc;
    if (!pp->ctl) {
        if ((rc = dalloc(&pp->ctl, CTL_WORDS))) return rc;
        CK(cudaMemset(pp->ctl, 0, sizeof(unsigned) * CTL_WORDS));
        int dev = 0, nsm = 1;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
        // one CTA per SM at most (the kernels' shared memory allows no more)
        pp->nblock = tune.grid > 0 ? std::min(tune.grid, nsm) : nsm;
        pp->ngene = n;
    }
    if (pp->ngene != n) return fail(GB_ERR_STATE, "persistent plan: gene count changed");
    // argument blocks (re-uploaded: buffers such as E may have been allocated since)
    std::vector<FastFwdArgs> fa(n);
    for (int k = 0; k < 2; k++) {
        for (int g = 0; g < n; g++) fa[g] = fwd_args(hs[g], k == 1);
        if (!pp->d_fargs[k] && (rc = dalloc(&pp->d_fargs[k], n))) return rc;
        CK(cudaMemcpy(pp->d_fargs[k], fa.data(), sizeof(FastFwdArgs) * n, cudaMemcpyHostToDevice));
    }
    if (!pp->d_ftask) {
        // children before parents.  Order 0 (critical path first): by depth
        // below the root, deepest first, all genes together, so that the nodes
        // with the longest chain of ancestors still to compute start first and
        // every gene's root comes in the last group; 1: gene by gene, level by
        // level (tree height); 2: level by level across genes
        std::vector<Task> t;
        auto push_level = [&](int g, int L) {
            const gb_handle *h = hs[g];
            if (L + 1 >= (int)h->level_off.size()) return;
            const int nt = h->npad / FAST_MT;
            for (int i = h->level_off[L]; i < h->level_off[L + 1]; i++)
                for (int tl = 0; tl < nt; tl++) t.push_back(Task{g, i, tl, 0});
        };
        int maxH = 0;
        for (int g = 0; g < n; g++) maxH = std::max(maxH, (int)hs[g]->level_off.size() - 1);
        if (tune.order == 1) {
            for (int g = 0; g < n; g++)
                for (int L = 0; L < maxH; L++) push_level(g, L);
        } else if (tune.order == 2) {
            for (int L = 0; L < maxH; L++)
                for (int g = 0; g < n; g++) push_level(g, L);
        } else {
            struct Key { int depth, g, i; };
            std::vector<Key> keys;
            for (int g = 0; g < n; g++) {
                const gb_handle *h = hs[g];
                for (int i = 0; i < (int)h->items.size(); i++) {
                    int d = 0;
                    for (int a = h->items[i].node; a != h->root; a = h->father[a]) d++;
                    keys.push_back(Key{d, g, i});
                }
            }
            std::stable_sort(keys.begin(), keys.end(), [](const Key &x, const Key &y) { return x.depth > y.depth; });
            for (const Key &k : keys) {
                const int nt = hs[k.g]->npad / FAST_MT;
                for (int tl = 0; tl < nt; tl++) t.push_back(Task{k.g, k.i, tl, 0});
            }
        }
        pp->nftask = (int)t.size();
        const char *tr = std::getenv("GBCODEML_TRACE");
        pp->tracing = tr && std::strcmp(tr, "1") == 0;
        if (pp->tracing && (rc = dalloc(&pp->trace[0], TRACE_WORDS * t.size()))) return rc;
        if ((rc = dalloc(&pp->d_ftask, t.size()))) return rc;
        CK(cudaMemcpy(pp->d_ftask, t.data(), sizeof(Task) * t.size(), cudaMemcpyHostToDevice));
    }
    if (!bwd) return 0;
    std::vector<FastBwdArgs> ba(n);
    for (int g = 0; g < n; g++) {
        if (!hs[g]->adj || !hs[g]->fast->ebexp) return fail(GB_ERR_STATE, "persistent plan: adjoint buffers missing");
        ba[g] = bwd_args(hs[g]);
    }
    if (!pp->d_bargs && (rc = dalloc(&pp->d_bargs, n))) return rc;
    CK(cudaMemcpy(pp->d_bargs, ba.data(), sizeof(FastBwdArgs) * n, cudaMemcpyHostToDevice));
    if (!pp->d_btask) {
        // parents before children: backward levels from each gene's root down
        std::vector<Task> t;
        auto push_item = [&](int g, int i) {
            // an item with two or more internal children (the root has three
            // children) is split into one task per child edge: each edge's
            // contractions are the bulk of the work, and near the root the
            // items are few
            const BItem &b = hs[g]->adj->bitems[i];
            const int nt = hs[g]->npad / FAST_MT;
            int ninternal = 0;
            for (int c = 0; c < b.nchild; c++) ninternal += b.tslot[c][0] >= 0;
            if (ninternal >= 2)
                for (int c = 0; c < b.nchild; c++)
                    for (int tl = 0; tl < nt; tl++) t.push_back(Task{g, i, tl, c});
            else
                for (int tl = 0; tl < nt; tl++) t.push_back(Task{g, i, tl, -1});
        };
        auto push_blevel = [&](int g, int d) {
            const AdjointState *ad = hs[g]->adj;
            if (d + 1 >= (int)ad->blevel_off.size()) return;
            for (int i = ad->blevel_off[d]; i < ad->blevel_off[d + 1]; i++) push_item(g, i);
        };
        int maxB = 0;
        for (int g = 0; g < n; g++) maxB = std::max(maxB, (int)hs[g]->adj->blevel_off.size() - 1);
        if (tune.order == 1) {
            for (int g = 0; g < n; g++)
                for (int d = 0; d < maxB; d++) push_blevel(g, d);
        } else if (tune.order == 2) {
            for (int d = 0; d < maxB; d++)
                for (int g = 0; g < n; g++) push_blevel(g, d);
        } else {
            // parents before children, critical path first: by the height of
            // the subtree below the node (the longest chain of descendants
            // still to compute), tallest first, all genes together
            struct Key { int height, g, i; };
            std::vector<Key> keys;
            for (int g = 0; g < n; g++) {
                const AdjointState *ad = hs[g]->adj;
                for (int i = 0; i < (int)ad->bitems.size(); i++)
                    keys.push_back(Key{hs[g]->height[ad->bitems[i].node], g, i});
            }
            std::stable_sort(keys.begin(), keys.end(), [](const Key &x, const Key &y) { return x.height > y.height; });
            for (const Key &k : keys) push_item(k.g, k.i);
        }
        pp->nbtask = (int)t.size();
        if (pp->tracing && (rc = dalloc(&pp->trace[1], TRACE_WORDS * t.size()))) return rc;
        if ((rc = dalloc(&pp->d_btask, t.size()))) return rc;
        CK(cudaMemcpy(pp->d_btask, t.data(), sizeof(Task) * t.size(), cudaMemcpyHostToDevice));
        // dlnL/dP: independent (gene, pair, chunk) tasks, heaviest first
        std::vector<std::pair<long, Task>> gt;
        for (int g = 0; g < n; g++) {
            const gb_handle *h = hs[g];
            const AdjointState *ad = h->adj;
            for (int p = 0; p < (int)h->pairs.size(); p++)
                for (int c = 0; c < ad->nchunk; c++) {
                    const long np = std::min(h->npatt, (c + 1) * ad->gchunk) - c * ad->gchunk;
                    gt.push_back({(long)(ad->coff[p + 1] - ad->coff[p]) * np, Task{g, p, c, 0}});
                }
        }
        std::stable_sort(gt.begin(), gt.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
        t.clear();
        for (auto &x : gt) t.push_back(x.second);
        pp->ngtask = (int)t.size();
        if (pp->tracing && (rc = dalloc(&pp->trace[2], TRACE_WORDS * t.size()))) return rc;
        if ((rc = dalloc(&pp->d_gtask, t.size()))) return rc;
        CK(cudaMemcpy(pp->d_gtask, t.data(), sizeof(Task) * t.size(), cudaMemcpyHostToDevice));
    }
    pp->has_bwd = true;
    return 0;
}

int persist_record_fwd(PersistPlan *pp, bool keepE, int ns, cudaStream_t st, gb_handle *prof) {
    launch_prune_persist(pp->d_fargs[keepE ? 1 : 0], pp->d_ftask, pp->nftask, pp->ctl, ns, pp->nblock,
                         pp->trace[0], st);
    if (prof) prof_mark(prof, GB_K_PRUNE);
    return 1;
}

int persist_record_bwd(PersistPlan *pp, int nsb, cudaStream_t st, gb_handle *prof) {
    launch_bwd_persist(pp->d_bargs, pp->d_btask, pp->nbtask, pp->ctl, nsb, pp->nblock, pp->trace[1], st);
    if (prof) prof_mark(prof, GB_K_BWD);
    launch_gradP_persist(pp->d_bargs, pp->d_gtask, pp->ngtask, pp->ctl, nsb, pp->nblock, pp->trace[2], st);
    if (prof) prof_mark(prof, GB_K_GRADP);
    return 2;
}

// ---------------------------------------------------------------- per-gene pieces

int fast_rec_pmat(gb_handle *h) {
    launch_pmat_fp64(h->d_pairs, (int)h->pairs.size(), h->d_label, h->d_tnode, h->d_prm, h->d_Pt, h->stream,
                     h->d_pi);
    prof_mark(h, GB_K_PMAT);
    FastFwdArgs a = fwd_args(h, false);
    launch_pslice(a, h->fast->ns, (int)h->pairs.size(), h->fast->umma, h->stream);
    prof_mark(h, GB_K_PMAT);
    return 2;
}

int fast_rec_mix(gb_handle *h) {
    // every node is renormalised, so fhK is always in log form
    launch_mix(h->d_fhK, h->d_fpatt, h->d_prm, h->npatt, h->npad, 1, h->d_lnf, h->d_post, h->d_partial,
               h->d_ticket, h->d_out, h->stream, h->d_fbar, h->fast->groot);
    prof_mark(h, GB_K_MIX);
    return 1;
}

int fast_rec_dmat(gb_handle *h) {
    launch_dmat(h);
    prof_mark(h, GB_K_OTHER);
    return 1;
}

int fast_rec_tail(gb_handle *h) {
    launch_gradH_df(h);
    prof_mark(h, GB_K_GRADH);
    launch_freq(h, 1);
    prof_mark(h, GB_K_OTHER);
    return 2;
}

int fast_rec_copies_in(gb_handle *h, bool grad) {
    CK(cudaMemcpyAsync(h->d_prm, h->h_prm, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->d_tnode, h->h_tnode, sizeof(double) * h->nnode, cudaMemcpyHostToDevice, h->stream));
    if (grad) CK(cudaMemcpyAsync(h->adj->d_gp, h->adj->h_gp, sizeof(GradParams), cudaMemcpyHostToDevice, h->stream));
    return 0;
}

int fast_rec_copies_out(gb_handle *h, bool grad) {
    if (grad) {
        int rc = adjoint_fetch(h);
        if (rc) return rc;
    }
    CK(cudaMemcpyAsync(h->h_out, h->d_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(h->fast->h_err, h->fast->err, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    return 0;
}

int fast_prepare(gb_handle *h, bool grad) {
    CK(cudaSetDevice(h->device));
    return fast_alloc(h, grad);
}

bool fast_persistent(const gb_handle *h) { return h->fast && h->fast->persist; }

float2 *fast_groot(gb_handle *h) { return h->fast ? h->fast->groot : nullptr; }

PsliceArgs fast_pslice_args(gb_handle *h) {
    FastState *f = h->fast;
    return PsliceArgs{h->d_Pt, f->Pdf, f->Bf, f->Bb};
}

void fast_swap_err(gb_handle *h, int *&d_err, int *&h_err) {
    std::swap(h->fast->err, d_err);
    std::swap(h->fast->h_err, h_err);
}

// the last evaluation's task trace of one persistent kernel of a plan:
// TRACE_OUT words per task (gene, item, tile, 0, then the kernel's TRACE_WORDS)
int persist_task_trace(PersistPlan *pp, int kernel, unsigned long long *out, int cap) {
    if (kernel < 0 || kernel > 2) return fail(GB_ERR_ARG, "task trace: kernel must be 0, 1 or 2");
    const Task *dt[3] = {pp->d_ftask, pp->d_btask, pp->d_gtask};
    const int nt[3] = {pp->nftask, pp->nbtask, pp->ngtask};
    if (!pp->tracing || !pp->trace[kernel] || !dt[kernel])
        return fail(GB_ERR_STATE, "task trace: tracing off (GBCODEML_TRACE=1 at creation) or kernel not run");
    const int n = std::min(cap, nt[kernel]);
    if (out && n > 0) {
        CK(cudaDeviceSynchronize());
        std::vector<Task> t(n);
        std::vector<unsigned long long> tr((size_t)TRACE_WORDS * n);
        CK(cudaMemcpy(t.data(), dt[kernel], sizeof(Task) * n, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(tr.data(), pp->trace[kernel], sizeof(unsigned long long) * TRACE_WORDS * n,
                      cudaMemcpyDeviceToHost));
        for (int i = 0; i < n; i++) {
            unsigned long long *o = out + (size_t)TRACE_OUT * i;
            o[0] = (unsigned long long)t[i].gene;
            o[1] = (unsigned long long)t[i].item;
            o[2] = (unsigned long long)t[i].tile;
            o[3] = (unsigned long long)(long long)t[i].edge;
            for (int q = 0; q < TRACE_WORDS; q++) o[4 + q] = tr[(size_t)TRACE_WORDS * i + q];
        }
    }
    return nt[kernel];
}

int fast_task_trace(gb_handle *h, int kernel, unsigned long long *out, int cap) {
    if (!h->fast || !h->fast->persist) return fail(GB_ERR_STATE, "gb_task_trace: no persistent kernels on this handle");
    CK(cudaSetDevice(h->device));
    return persist_task_trace(&h->fast->plan, kernel, out, cap);
}
int fast_fault_inject(gb_handle *h, int wait_ms, int withhold) {
    if (!h->fast || !h->fast->persist || !h->fast->plan.ctl)
        return fail(GB_ERR_STATE, "gb_fault_inject: the handle's persistent kernels have not run yet");
    if (wait_ms < 0 || wait_ms > 60000 || (withhold != 0 && withhold != 1))
        return fail(GB_ERR_ARG, "gb_fault_inject: wait_ms in 0..60000, withhold 0 or 1");
    CK(cudaSetDevice(h->device));
    CK(cudaStreamSynchronize(h->stream));
    const unsigned w[2] = {(unsigned)withhold, (unsigned)wait_ms};
    CK(cudaMemcpy(h->fast->plan.ctl + CTL_SKEW, w, sizeof(w), cudaMemcpyHostToDevice));
    return GB_OK;
}
int fast_ns(const gb_handle *h, bool adjoint) { return adjoint ? h->fast->nsb : h->fast->ns; }

// one gene's whole evaluation with one launch per tree level (batches whose
// genes do not share a persistent plan)
int fast_record_eval(gb_handle *h, bool grad) {
    int rc = fast_rec_copies_in(h, grad);
    if (rc) return rc;
    int nk = fast_rec_pmat(h) + rec_levels_fwd(h, grad) + fast_rec_mix(h);
    if (grad) nk += fast_rec_dmat(h) + rec_levels_bwd(h) + fast_rec_tail(h);
    if ((rc = fast_rec_copies_out(h, grad))) return rc;
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
    h->h_prm->sym = D->sym;
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
