// Batched evaluation of many independent alignments (genes): one handle per
// gene, and ONE CUDA graph per batch evaluation.  Split precision with the
// persistent kernels: the pruning recursion, the adjoint propagation and
// dlnL/dP of ALL genes are one persistent launch each over a task list that
// mixes the genes (tasks in critical-path order, dependencies tracked per
// (slot, tile) on the device), and the small per-gene steps (P matrices and
// their digit planes, the mixture, dP/dt, per-pair sums) are one launch each
// over all genes (a block-to-gene map); the genes' per-evaluation inputs and
// results live in batch-wide staging buffers, so each is one copy.  Otherwise
// (FP64, or genes without a shared persistent plan) every gene's whole
// evaluation is an independent graph branch.  The host side (eigen solutions, Qfactors, chain rule of
// the gradient) runs on a pool of host threads, one slice of genes per thread.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "adjoint_internal.h"
#include "batch_internal.h"
#include "fast_internal.h"
#include "handle.h"

struct gb_batch {
    int n = 0, precision = 0, device = 0, nthreads = 1;
    std::vector<gb_handle *> h;
    std::vector<gb::Derived *> D;
    cudaStream_t origin = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, fork = nullptr;
    std::vector<cudaEvent_t> join;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int kernels[2] = {0, 0};
    gb::PersistPlan plan;
    gb::Tuning tune;
    // batch-wide staging of per-evaluation inputs / results (persistent path);
    // each gene's handle points into them (its own buffers are swapped out and
    // swapped back before it is destroyed)
    struct Staging {
        bool base = false, adj = false;
        gb::DevParams *d_prm = nullptr, *h_prm = nullptr;
        double *d_tnode = nullptr, *h_tnode = nullptr;
        double *d_out = nullptr, *h_out = nullptr;
        int *d_err = nullptr, *h_err = nullptr;
        gb::GradParams *d_gp = nullptr, *h_gp = nullptr;
        double *d_pout = nullptr, *h_pout = nullptr, *d_fpart = nullptr, *h_fpart = nullptr;
        size_t ntnode = 0, npout = 0, nfpart = 0;
        std::vector<gb::DevParams *> sv_dprm, sv_hprm;
        std::vector<double *> sv_dt, sv_ht, sv_dout, sv_hout, sv_dpout, sv_hpout, sv_dfp, sv_hfp;
        std::vector<int *> sv_derr, sv_herr;
        std::vector<gb::GradParams *> sv_dgp, sv_hgp;
    } st;
    // batched launches: per-gene argument blocks and block-to-gene maps
    struct Launch {
        void *args = nullptr;
        int2 *map = nullptr;
        int nblocks = 0;
    } l_pmat, l_pslice, l_mix, l_mixg, l_dmat, l_gradH, l_freq;   // l_mixg: with the adjoint's root seed
    // an evaluation submitted and not yet collected (gb_batch_submit / _collect)
    bool pending = false, pending_grad = false;
    double pending_t0 = 0;
    std::vector<std::vector<double>> pending_blength;
};

namespace {

using namespace gb;

template <class F>
void parallel_for(int n, int nthreads, F fn) {
    nthreads = std::max(1, std::min(nthreads, n));
    if (nthreads == 1) {
        for (int i = 0; i < n; i++) fn(i);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; t++)
        th.emplace_back([&, t] {
            for (int i = t; i < n; i += nthreads) fn(i);
        });
    for (auto &x : th) x.join();
}

void unstage(gb_batch *b);

void free_launch(gb_batch::Launch &l) {
    if (l.args) cudaFree(l.args);
    if (l.map) cudaFree(l.map);
    l = gb_batch::Launch();
}

void batch_free(gb_batch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
    unstage(b);
    for (auto *l : {&b->l_pmat, &b->l_pslice, &b->l_mix, &b->l_mixg, &b->l_dmat, &b->l_gradH, &b->l_freq})
        free_launch(*l);
    for (auto &g : b->graph)
        if (g) cudaGraphExecDestroy(g);
    for (auto e : b->join)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->origin) cudaStreamDestroy(b->origin);
    gb::persist_free(&b->plan);
    for (auto h : b->h)
        if (h) gb_destroy(h);
    for (auto d : b->D) delete d;
    delete b;
}

// ---------------------------------------------------------------- staging

template <class T>
int hstage(T **p, size_t n) {
    if (cudaMallocHost((void **)p, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) {
        *p = nullptr;
        return fail(GB_ERR_OOM, "batch staging: cudaMallocHost");
    }
    std::memset(*p, 0, sizeof(T) * std::max<size_t>(n, 1));
    return 0;
}

// point every gene's parameter, branch-length and result buffers into the
// batch-wide ones (adj: also the gradient inputs and per-pair / class sums)
int stage(gb_batch *b, bool adj) {
    auto &s = b->st;
    int rc;
    const int n = b->n;
    if (!s.base) {
        s.ntnode = 0;
        for (auto h : b->h) s.ntnode += h->nnode;
        if ((rc = dalloc(&s.d_prm, n)) || (rc = hstage(&s.h_prm, n)) || (rc = dalloc(&s.d_tnode, s.ntnode)) ||
            (rc = hstage(&s.h_tnode, s.ntnode)) || (rc = dalloc(&s.d_out, 4 * (size_t)n)) ||
            (rc = hstage(&s.h_out, 4 * (size_t)n)) || (rc = dalloc(&s.d_err, n)) || (rc = hstage(&s.h_err, n)))
            return rc;
        CK(cudaMemset(s.d_err, 0, sizeof(int) * n));
        size_t off = 0;
        for (int i = 0; i < n; i++) {
            gb_handle *h = b->h[i];
            // keep what the host already staged for the next evaluation
            std::memcpy(s.h_prm + i, h->h_prm, sizeof(DevParams));
            std::memcpy(s.h_tnode + off, h->h_tnode, sizeof(double) * h->nnode);
            s.sv_dprm.push_back(h->d_prm), s.sv_hprm.push_back(h->h_prm);
            s.sv_dt.push_back(h->d_tnode), s.sv_ht.push_back(h->h_tnode);
            s.sv_dout.push_back(h->d_out), s.sv_hout.push_back(h->h_out);
            h->d_prm = s.d_prm + i;
            h->h_prm = s.h_prm + i;
            h->d_tnode = s.d_tnode + off;
            h->h_tnode = s.h_tnode + off;
            h->d_out = s.d_out + 4 * (size_t)i;
            h->h_out = s.h_out + 4 * (size_t)i;
            int *de = s.d_err + i, *he = s.h_err + i;
            fast_swap_err(h, de, he);
            s.sv_derr.push_back(de), s.sv_herr.push_back(he);
            off += h->nnode;
        }
        s.base = true;
    }
    if (adj && !s.adj) {
        s.npout = s.nfpart = 0;
        for (auto h : b->h) {
            if (!h->adj) return fail(GB_ERR_STATE, "batch staging: adjoint buffers missing");
            s.npout += h->pairs.size() * 3;
            s.nfpart += (size_t)h->adj->nfreq_blocks * 4;
        }
        if ((rc = dalloc(&s.d_gp, n)) || (rc = hstage(&s.h_gp, n)) || (rc = dalloc(&s.d_pout, s.npout)) ||
            (rc = hstage(&s.h_pout, s.npout)) || (rc = dalloc(&s.d_fpart, s.nfpart)) ||
            (rc = hstage(&s.h_fpart, s.nfpart)))
            return rc;
        size_t op = 0, of = 0;
        for (int i = 0; i < n; i++) {
            AdjointState *a = b->h[i]->adj;
            std::memcpy(s.h_gp + i, a->h_gp, sizeof(GradParams));
            s.sv_dgp.push_back(a->d_gp), s.sv_hgp.push_back(a->h_gp);
            s.sv_dpout.push_back(a->d_pout), s.sv_hpout.push_back(a->h_pout);
            s.sv_dfp.push_back(a->d_fpart), s.sv_hfp.push_back(a->h_fpart);
            a->d_gp = s.d_gp + i;
            a->h_gp = s.h_gp + i;
            a->d_pout = s.d_pout + op;
            a->h_pout = s.h_pout + op;
            a->d_fpart = s.d_fpart + of;
            a->h_fpart = s.h_fpart + of;
            op += b->h[i]->pairs.size() * 3;
            of += (size_t)a->nfreq_blocks * 4;
        }
        s.adj = true;
    }
    return 0;
}

void unstage(gb_batch *b) {
    auto &s = b->st;
    for (int i = 0; i < (int)s.sv_dprm.size(); i++) {
        gb_handle *h = b->h[i];
        h->d_prm = s.sv_dprm[i], h->h_prm = s.sv_hprm[i];
        h->d_tnode = s.sv_dt[i], h->h_tnode = s.sv_ht[i];
        h->d_out = s.sv_dout[i], h->h_out = s.sv_hout[i];
        fast_swap_err(h, s.sv_derr[i], s.sv_herr[i]);
    }
    for (int i = 0; i < (int)s.sv_dgp.size(); i++) {
        AdjointState *a = b->h[i]->adj;
        a->d_gp = s.sv_dgp[i], a->h_gp = s.sv_hgp[i];
        a->d_pout = s.sv_dpout[i], a->h_pout = s.sv_hpout[i];
        a->d_fpart = s.sv_dfp[i], a->h_fpart = s.sv_hfp[i];
    }
    void *dv[] = {s.d_prm, s.d_tnode, s.d_out, s.d_err, s.d_gp, s.d_pout, s.d_fpart};
    for (void *p : dv)
        if (p) cudaFree(p);
    void *hv[] = {s.h_prm, s.h_tnode, s.h_out, s.h_err, s.h_gp, s.h_pout, s.h_fpart};
    for (void *p : hv)
        if (p) cudaFreeHost(p);
    s = gb_batch::Staging();
}

// ---------------------------------------------------------------- batched launches

// built once: captured graphs keep pointing at these arrays
template <class A, class F>
int make_launch(gb_batch *b, gb_batch::Launch &l, F per_gene) {   // per_gene(h, &args) -> blocks
    if (l.args) return 0;
    std::vector<A> args(b->n);
    std::vector<int2> map;
    for (int g = 0; g < b->n; g++) {
        const int nb = per_gene(b->h[g], &args[g]);
        for (int j = 0; j < nb; j++) map.push_back(make_int2(g, j));
    }
    int rc;
    A *da = nullptr;
    if ((rc = dalloc(&da, args.size())) || (rc = dalloc(&l.map, map.size()))) return rc;
    l.args = da;
    CK(cudaMemcpy(da, args.data(), sizeof(A) * args.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(l.map, map.data(), sizeof(int2) * std::max<size_t>(map.size(), 1), cudaMemcpyHostToDevice));
    l.nblocks = (int)map.size();
    return 0;
}

int build_launches(gb_batch *b, bool grad) {
    int rc;
    if ((rc = make_launch<PmatArgs>(b, b->l_pmat, [](gb_handle *h, PmatArgs *a) {
             *a = PmatArgs{h->d_pairs, h->d_label, h->d_tnode, h->d_prm, h->d_Pt, h->d_pi};
             return (int)h->pairs.size();
         })) ||
        (rc = make_launch<PsliceArgs>(b, b->l_pslice, [](gb_handle *h, PsliceArgs *a) {
             *a = fast_pslice_args(h);
             return (int)h->pairs.size();
         })) ||
        (rc = make_launch<MixArgs>(b, grad ? b->l_mixg : b->l_mix, [grad](gb_handle *h, MixArgs *a) {
             const int nb = (h->npatt + 255) / 256;
             *a = MixArgs{h->d_fhK, h->d_fpatt, h->d_prm, h->npatt, h->npad, 1, nb,
                          h->d_lnf, h->d_post, h->d_partial, h->d_ticket, h->d_out, h->d_fbar,
                          grad ? fast_groot(h) : nullptr};
             return nb;
         })))
        return rc;
    if (!grad) return 0;
    if ((rc = make_launch<DmatArgs>(b, b->l_dmat, [](gb_handle *h, DmatArgs *a) {
             *a = DmatArgs{h->d_prm, h->adj->d_gp, h->adj->d_Dm, h->adj->d_UVdf};
             return DM_BLOCKS;
         })) ||
        (rc = make_launch<GradHArgs>(b, b->l_gradH, [](gb_handle *h, GradHArgs *a) {
             AdjointState *ad = h->adj;
             *a = GradHArgs{h->d_pairs, h->d_label, h->d_tnode, h->d_prm,
                            reinterpret_cast<const float2 *>(ad->d_Gpart), ad->nchunk, ad->d_Dm, ad->d_UVdf,
                            ad->d_pout};
             return (int)h->pairs.size();
         })) ||
        (rc = make_launch<FreqArgs>(b, b->l_freq, [](gb_handle *h, FreqArgs *a) {
             *a = FreqArgs{h->d_fhK, h->d_lnf, h->d_fpatt, h->npatt, h->npad, 1, h->adj->d_fpart};
             return h->adj->nfreq_blocks;
         })))
        return rc;
    return 0;
}

// every gene's branch: origin -> gene stream -> fn(h) -> origin
template <class F>
int fork_join(gb_batch *b, F fn) {
    CK(cudaEventRecord(b->fork, b->origin));
    int nk = 0;
    for (int i = 0; i < b->n; i++) {
        gb_handle *h = b->h[i];
        CK(cudaStreamWaitEvent(h->stream, b->fork, 0));
        const int r = fn(h);
        if (r < 0) return r;
        nk += r;
        CK(cudaEventRecord(b->join[i], h->stream));
        CK(cudaStreamWaitEvent(b->origin, b->join[i], 0));
    }
    return nk;
}

bool batch_persistent(const gb_batch *b) {
    for (auto h : b->h)
        if (h->precision != GB_PREC_FAST || !fast_persistent(h) || fast_ns(h, false) != fast_ns(b->h[0], false) ||
            fast_ns(h, true) != fast_ns(b->h[0], true))
            return false;
    return true;
}

int record_persistent(gb_batch *b, bool grad) {
    const int ns = fast_ns(b->h[0], false), nsb = fast_ns(b->h[0], true);
    auto &s = b->st;
    cudaStream_t o = b->origin;
    launch_bump(b->plan.ctl, o);
    CK(cudaMemcpyAsync(s.d_prm, s.h_prm, sizeof(DevParams) * b->n, cudaMemcpyHostToDevice, o));
    CK(cudaMemcpyAsync(s.d_tnode, s.h_tnode, sizeof(double) * s.ntnode, cudaMemcpyHostToDevice, o));
    if (grad) CK(cudaMemcpyAsync(s.d_gp, s.h_gp, sizeof(GradParams) * b->n, cudaMemcpyHostToDevice, o));
    launch_pmat_batched((const PmatArgs *)b->l_pmat.args, b->l_pmat.map, b->l_pmat.nblocks, o);
    launch_pslice_batched((const PsliceArgs *)b->l_pslice.args, b->l_pslice.map, b->l_pslice.nblocks, ns, o);
    int nk = 3 + persist_record_fwd(&b->plan, grad, ns, o, nullptr);
    const gb_batch::Launch &lm = grad ? b->l_mixg : b->l_mix;
    launch_mix_batched((const MixArgs *)lm.args, lm.map, lm.nblocks, o);
    nk++;
    if (grad) {
        launch_dmat_batched((const DmatArgs *)b->l_dmat.args, b->l_dmat.map, b->l_dmat.nblocks, o);
        nk += 1 + persist_record_bwd(&b->plan, nsb, o, nullptr);
        launch_gradH_batched((const GradHArgs *)b->l_gradH.args, b->l_gradH.map, b->l_gradH.nblocks, o);
        launch_freq_batched((const FreqArgs *)b->l_freq.args, b->l_freq.map, b->l_freq.nblocks, o);
        nk += 2;
        CK(cudaMemcpyAsync(s.h_pout, s.d_pout, sizeof(double) * s.npout, cudaMemcpyDeviceToHost, o));
        CK(cudaMemcpyAsync(s.h_fpart, s.d_fpart, sizeof(double) * s.nfpart, cudaMemcpyDeviceToHost, o));
    }
    CK(cudaMemcpyAsync(s.h_out, s.d_out, sizeof(double) * 4 * b->n, cudaMemcpyDeviceToHost, o));
    CK(cudaMemcpyAsync(s.h_err, s.d_err, sizeof(int) * b->n, cudaMemcpyDeviceToHost, o));
    return nk;
}

int build_graph(gb_batch *b, bool grad) {
    cudaGraphExec_t &ge = b->graph[grad ? 1 : 0];
    if (ge) return 0;
    for (auto h : b->h) {
        int rc = h->precision == GB_PREC_FAST ? fast_prepare(h, grad) : fp64_prepare(h, grad);
        if (rc) return rc;
    }
    const bool persist = batch_persistent(b);
    if (persist) {
        int rc;
        if ((rc = stage(b, grad)) || (rc = persist_build(&b->plan, b->h.data(), b->n, grad, b->tune)) ||
            (rc = build_launches(b, grad)))
            return rc;
    }
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(b->origin, cudaStreamCaptureModeThreadLocal));
    int nk;
    if (persist) {
        nk = record_persistent(b, grad);
    } else {
        nk = fork_join(b, [&](gb_handle *h) {
            return h->precision == GB_PREC_FAST ? fast_record_eval(h, grad) : fp64_record_eval(h, grad);
        });
    }
    if (nk < 0) {
        cudaStreamEndCapture(b->origin, &g);
        if (g) cudaGraphDestroy(g);
        return nk;
    }
    CK(cudaStreamEndCapture(b->origin, &g));
    cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (batch)");
    b->kernels[grad ? 1 : 0] = nk;
    return 0;
}

}  // namespace

extern "C" {

int gb_batch_create(int ngene, const gb_problem *probs, gb_batch **out) {
    if (ngene < 1 || !probs || !out) return fail(GB_ERR_ARG, "gb_batch_create: bad arguments");
    *out = nullptr;
    gb_batch *b = new gb_batch();
    b->n = ngene;
    b->precision = probs[0].precision;
    b->device = probs[0].device;
    b->nthreads = std::max(1u, std::thread::hardware_concurrency());
    b->h.assign(ngene, nullptr);
    b->D.assign(ngene, nullptr);
    for (int i = 0; i < ngene; i++) {
        if (probs[i].device != b->device) { batch_free(b); return fail(GB_ERR_ARG, "gb_batch_create: one device per batch"); }
        int rc = gb_create(&probs[i], &b->h[i]);
        if (rc) { batch_free(b); return rc; }
        // a batch's dlnL/dP tasks come from all genes: the long chunks need no
        // per-gene adjustment (gb_batch_tune may still set another)
        b->h[i]->tune.gchunk = GCHUNK_FAST;
        b->D[i] = new Derived;
    }
    if (cudaSetDevice(b->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->origin, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
        batch_free(b);
        return fail(GB_ERR_CUDA, "gb_batch_create: stream/event creation");
    }
    b->join.assign(ngene, nullptr);
    for (auto &e : b->join)
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
            batch_free(b);
            return fail(GB_ERR_CUDA, "gb_batch_create: event creation");
        }
    *out = b;
    return GB_OK;
}

int gb_batch_destroy(gb_batch *b) {
    if (!b) return fail(GB_ERR_STATE, "null batch");
    batch_free(b);
    return GB_OK;
}

int gb_batch_size(const gb_batch *b) { return b ? b->n : GB_ERR_STATE; }

namespace {
// gb_batch_submit and gb_batch_submit_b: omega1 (nullable) gives each gene
// branch-site model B's free w1 (model A: w1 = 1)
int batch_submit(gb_batch *b, const gb_params *prm, const double *omega1, int with_grad, const gb_batch *after) {
    if (!b || !prm) return fail(GB_ERR_ARG, "gb_batch_submit: bad arguments");
    if (b->pending) return fail(GB_ERR_STATE, "gb_batch_submit: the previous evaluation was not collected");
    if (after && after->device != b->device) return fail(GB_ERR_ARG, "gb_batch_submit: batches on two devices");
    const bool grad = with_grad != 0;
    CK(cudaSetDevice(b->device));
    const double t0 = now_ms();
    // host: model set-up of every gene, in parallel
    std::vector<int> status(b->n, 0);
    parallel_for(b->n, b->nthreads, [&](int i) {
        gb_handle *h = b->h[i];
        ModelParams m{prm[i].kappa, prm[i].omega0, prm[i].omega2, prm[i].p0, prm[i].p1};
        if (omega1) {
            m.w1 = omega1[i];
            m.free_w1 = true;
        }
        int rc = prm[i].blength ? derive(h->pi.data(), m, grad, b->D[i], false) : GB_ERR_ARG;
        if (!rc) rc = stage_params(h, b->D[i], prm[i].blength);
        status[i] = rc;
    });
    for (int i = 0; i < b->n; i++)
        if (status[i]) return fail(status[i], "gb_batch_eval: gene " + std::to_string(i) + ": parameters out of range");
    if (grad) {
        for (int i = 0; i < b->n; i++)
            if (!b->h[i]->adj) {
                int rc = adjoint_init(b->h[i]);
                if (rc) return rc;
            }
        b->pending_blength.resize(b->n);
        parallel_for(b->n, b->nthreads, [&](int i) {
            std::memcpy(b->h[i]->adj->h_gp->dQk, b->D[i]->dQk, sizeof(b->D[i]->dQk));
            std::memcpy(b->h[i]->adj->h_gp->dQw, b->D[i]->dQw, sizeof(b->D[i]->dQw));
            b->pending_blength[i].assign(prm[i].blength, prm[i].blength + b->h[i]->nnode);
        });
    }
    int rc = build_graph(b, grad);
    if (rc) return rc;
    // another batch's evaluation first (its graph's end event), so that the
    // device runs the two back to back while the host prepares the next
    if (after && after->ev1) CK(cudaStreamWaitEvent(b->origin, after->ev1, 0));
    CK(cudaEventRecord(b->ev0, b->origin));
    CK(cudaGraphLaunch(b->graph[grad ? 1 : 0], b->origin));
    CK(cudaEventRecord(b->ev1, b->origin));
    b->pending = true;
    b->pending_grad = grad;
    b->pending_t0 = t0;
    return GB_OK;
}
}  // namespace

int gb_batch_submit(gb_batch *b, const gb_params *prm, int with_grad, const gb_batch *after) {
    return batch_submit(b, prm, nullptr, with_grad, after);
}

int gb_batch_submit_b(gb_batch *b, const gb_params *prm, const double *omega1, int with_grad,
                      const gb_batch *after) {
    if (!omega1) return fail(GB_ERR_ARG, "gb_batch_submit_b: null omega1");
    return batch_submit(b, prm, omega1, with_grad, after);
}

int gb_batch_collect(gb_batch *b, double *neg_lnL, gb_grad *grads, gb_stats *stats) {
    if (!b || !neg_lnL) return fail(GB_ERR_ARG, "gb_batch_collect: bad arguments");
    if (!b->pending) return fail(GB_ERR_STATE, "gb_batch_collect: nothing submitted");
    const bool grad = b->pending_grad;
    if (grads && !grad) return fail(GB_ERR_ARG, "gb_batch_collect: the evaluation was submitted without gradient");
    b->pending = false;
    CK(cudaSetDevice(b->device));
    CK(cudaStreamSynchronize(b->origin));
    CK(cudaGetLastError());
    int rc;
    for (int i = 0; i < b->n; i++)
        if (b->h[i]->precision == GB_PREC_FAST && (rc = fast_check_error(b->h[i]))) return rc;
    for (int i = 0; i < b->n; i++) neg_lnL[i] = b->h[i]->h_out[0];
    if (grads)
        parallel_for(b->n, b->nthreads, [&](int i) {
            adjoint_chain(b->h[i], b->D[i], b->pending_blength[i].data(), &grads[i]);
        });
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        stats->ms_device = ms;
        stats->ms_host = now_ms() - b->pending_t0;
        stats->kernels = b->kernels[grad ? 1 : 0];
        stats->nscale = 0;
        double h2d = 0, d2h = 0;
        for (auto h : b->h) {
            h2d += sizeof(DevParams) + sizeof(double) * h->nnode + (grad ? sizeof(GradParams) : 0);
            d2h += sizeof(double) + (h->precision == GB_PREC_FAST ? sizeof(int) : 0) +
                   (grad ? sizeof(double) * (h->pairs.size() * 3 + h->adj->nfreq_blocks * 4) : 0);
        }
        stats->h2d_bytes = h2d;
        stats->d2h_bytes = d2h;
    }
    return GB_OK;
}

int gb_batch_omega1_grad(const gb_batch *b, double *d_omega1) {
    if (!b || !d_omega1) return fail(GB_ERR_ARG, "gb_batch_omega1_grad: bad arguments");
    for (int i = 0; i < b->n; i++) {
        if (!b->h[i]->adj) return fail(GB_ERR_STATE, "gb_batch_omega1_grad: no gradient collected");
        d_omega1[i] = b->h[i]->adj->d_omega1;
    }
    return GB_OK;
}

int gb_batch_eval(gb_batch *b, const gb_params *prm, double *neg_lnL, gb_grad *grads, gb_stats *stats) {
    if (!b || !prm || !neg_lnL) return fail(GB_ERR_ARG, "gb_batch_eval: bad arguments");
    int rc = gb_batch_submit(b, prm, grads != nullptr, nullptr);
    if (rc) return rc;
    return gb_batch_collect(b, neg_lnL, grads, stats);
}

int gb_batch_tune(gb_batch *b, int knob, int value) {
    if (!b) return fail(GB_ERR_ARG, "gb_batch_tune: null batch");
    if (b->graph[0] || b->graph[1] || b->plan.ctl) return fail(GB_ERR_STATE, "gb_batch_tune: batch already evaluated");
    if (knob == GB_TUNE_ORDER) {
        if (value < 0 || value > 2) return fail(GB_ERR_ARG, "gb_batch_tune: order must be 0, 1 or 2");
        b->tune.order = value;
        return GB_OK;
    }
    for (auto h : b->h) {
        const int rc = gb_tune(h, knob, value);
        if (rc) return rc;
    }
    if (knob == GB_TUNE_GRID) b->tune.grid = value;
    return GB_OK;
}

int gb_batch_task_trace(gb_batch *b, int kernel, unsigned long long *out, int cap) {
    if (!b || cap < 0) return fail(GB_ERR_ARG, "gb_batch_task_trace: bad arguments");
    if (!b->plan.ctl) return fail(GB_ERR_STATE, "gb_batch_task_trace: the batch has no persistent kernels");
    CK(cudaSetDevice(b->device));
    return persist_task_trace(&b->plan, kernel, out, cap);
}

int gb_batch_replay(gb_batch *b, int iters, int with_grad, double *ms) {
    if (!b || !ms || iters < 1) return fail(GB_ERR_ARG, "gb_batch_replay: bad arguments");
    cudaGraphExec_t g = b->graph[with_grad ? 1 : 0];
    if (!g) return fail(GB_ERR_STATE, "gb_batch_replay: evaluate first");
    CK(cudaSetDevice(b->device));
    CK(cudaEventRecord(b->ev0, b->origin));
    for (int i = 0; i < iters; i++) CK(cudaGraphLaunch(g, b->origin));
    CK(cudaEventRecord(b->ev1, b->origin));
    CK(cudaStreamSynchronize(b->origin));
    float t = 0;
    CK(cudaEventElapsedTime(&t, b->ev0, b->ev1));
    *ms = t;
    return GB_OK;
}

}  // extern "C"
