// Batched evaluation of many independent alignments (genes): one handle per
// gene, and ONE CUDA graph per batch evaluation.  Split precision with the
// persistent kernels: the pruning recursion, the adjoint propagation and
// dlnL/dP of ALL genes are one persistent launch each over a task list that
// mixes the genes (tasks ordered by tree level, dependencies tracked per
// (slot, tile) on the device); the small per-gene steps (P matrices and their
// digit planes, the mixture, dP/dt, per-pair sums, copies) are independent
// graph branches between them.  Otherwise every gene's whole evaluation is an
// independent branch.  The host side (eigen solutions, Qfactors, chain rule of
// the gradient) runs on a pool of host threads, one slice of genes per thread.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "adjoint_internal.h"
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

void batch_free(gb_batch *b) {
    if (!b) return;
    cudaSetDevice(b->device);
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
    launch_bump(b->plan.ctl, b->origin);
    int nk = 1, r;
    if ((r = fork_join(b, [&](gb_handle *h) {
             const int rc = fast_rec_copies_in(h, grad);
             return rc ? rc : fast_rec_pmat(h);
         })) < 0)
        return r;
    nk += r + persist_record_fwd(&b->plan, grad, ns, b->origin, nullptr);
    if ((r = fork_join(b, [&](gb_handle *h) { return fast_rec_mix(h) + (grad ? fast_rec_dmat(h) : 0); })) < 0)
        return r;
    nk += r;
    if (grad) nk += persist_record_bwd(&b->plan, nsb, b->origin, nullptr);
    if ((r = fork_join(b, [&](gb_handle *h) {
             const int n = grad ? fast_rec_tail(h) : 0;
             const int rc = fast_rec_copies_out(h, grad);
             return rc ? rc : n;
         })) < 0)
        return r;
    return nk + r;
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
        int rc = persist_build(&b->plan, b->h.data(), b->n, grad, b->tune);
        if (rc) return rc;
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

int gb_batch_eval(gb_batch *b, const gb_params *prm, double *neg_lnL, gb_grad *grads, gb_stats *stats) {
    if (!b || !prm || !neg_lnL) return fail(GB_ERR_ARG, "gb_batch_eval: bad arguments");
    const bool grad = grads != nullptr;
    CK(cudaSetDevice(b->device));
    const double t0 = now_ms();
    // host: model set-up of every gene, in parallel
    std::vector<int> status(b->n, 0);
    parallel_for(b->n, b->nthreads, [&](int i) {
        gb_handle *h = b->h[i];
        ModelParams m{prm[i].kappa, prm[i].omega0, prm[i].omega2, prm[i].p0, prm[i].p1};
        int rc = prm[i].blength ? derive(h->pi.data(), m, grad, b->D[i]) : GB_ERR_ARG;
        if (!rc) rc = stage_params(h, b->D[i], prm[i].blength);
        status[i] = rc;
    });
    for (int i = 0; i < b->n; i++)
        if (status[i]) return fail(status[i], "gb_batch_eval: gene " + std::to_string(i) + ": parameters out of range");
    if (grad)
        for (int i = 0; i < b->n; i++) {
            if (!b->h[i]->adj) {
                int rc = adjoint_init(b->h[i]);
                if (rc) return rc;
            }
            std::memcpy(b->h[i]->adj->h_gp->dQk, b->D[i]->dQk, sizeof(b->D[i]->dQk));
            std::memcpy(b->h[i]->adj->h_gp->dQw, b->D[i]->dQw, sizeof(b->D[i]->dQw));
        }
    int rc = build_graph(b, grad);
    if (rc) return rc;
    CK(cudaEventRecord(b->ev0, b->origin));
    CK(cudaGraphLaunch(b->graph[grad ? 1 : 0], b->origin));
    CK(cudaEventRecord(b->ev1, b->origin));
    CK(cudaStreamSynchronize(b->origin));
    CK(cudaGetLastError());
    for (int i = 0; i < b->n; i++)
        if (b->h[i]->precision == GB_PREC_FAST && (rc = fast_check_error(b->h[i]))) return rc;
    for (int i = 0; i < b->n; i++) neg_lnL[i] = b->h[i]->h_out[0];
    if (grad) parallel_for(b->n, b->nthreads, [&](int i) { adjoint_chain(b->h[i], b->D[i], prm[i].blength, &grads[i]); });
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, b->ev0, b->ev1);
        stats->ms_device = ms;
        stats->ms_host = now_ms() - t0;
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

int gb_batch_tune(gb_batch *b, int knob, int value) {
    if (!b) return fail(GB_ERR_ARG, "gb_batch_tune: null batch");
    if (b->graph[0] || b->graph[1] || b->plan.ctl) return fail(GB_ERR_STATE, "gb_batch_tune: batch already evaluated");
    if (knob == GB_TUNE_ORDER) {
        if (value != 0 && value != 1) return fail(GB_ERR_ARG, "gb_batch_tune: order must be 0 or 1");
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
