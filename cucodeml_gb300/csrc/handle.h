// The handle (gb_handle) and helpers shared by the host-side modules of the
// library: runtime.cu (schedule, forward), adjoint.cu (gradient) and fast.cu
// (split-precision path).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gbcodeml.h"
#include "internal.h"
#include "model.h"

namespace gb {

struct AdjointState;
struct CladeState;
struct FastState;
struct PersistPlan;

int fail(int code, const std::string &msg);
double now_ms();
int cuda_fail(cudaError_t e, const char *what);

template <class T>
int dalloc(T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, "cudaMalloc");
    }
    return 0;
}

#define CK(call)                                     \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return ::gb::cuda_fail(e_, #call); \
    } while (0)

int adjoint_run(gb_handle *h, const Derived *D, const ModelParams &m, const double *blength,
                gb_grad *grad, gb_stats *stats);
int adjoint_record(gb_handle *h);          // backward launches on h->stream (profiling)
int adjoint_launch_graph(gb_handle *h);    // replay the captured backward graph
bool adjoint_ready(gb_handle *h);

// profiling: when h->prof is set, launch sites call prof_mark after each kernel
struct ProfRec {
    std::vector<cudaEvent_t> ev;
    std::vector<int> cls;
};
void prof_mark(gb_handle *h, int cls);
void adjoint_free(AdjointState *a);
void clade_free(CladeState *c);
int fast_eval(gb_handle *h, const Derived *D, const double *blength, double *neg_lnL, gb_grad *grad,
              double *fhK, double *lnf, gb_stats *stats);
int fast_replay(gb_handle *h, int iters, int with_grad, double *ms);
int fast_profile(gb_handle *h, int iters, int with_grad, double *ms, int *launches);
void fast_free(FastState *f);

}  // namespace gb

namespace gb {
struct Tuning {                     // gb_tune knobs; -1 / 0: default
    int mma = -1, persist = -1, gchunk = 0, order = 0, grid = 0;
    int checkpoint = 0;              // FP64 adjoint: edge messages recomputed per level
};
}  // namespace gb

struct gb_handle {
    int device = 0;
    gb::Tuning tune;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int ns = 0, nnode = 0, root = 0, npatt = 0, npad = 0, ntile = 0, precision = 0;
    int fast_slices = 8;            // digit planes per operand in the split-precision path
    std::vector<int> father, label, nson, sons, height, dirty;
    std::vector<char> scale;
    std::vector<double> pi, fpatt;
    int nscale = 0;

    // schedule
    std::vector<gb::Item> items;        // grouped by level
    std::vector<int> level_off;     // items of level L: [level_off[L], level_off[L+1])
    std::vector<gb::PairDesc> pairs;
    std::vector<int> pair_of;       // [nnode*3] pair index of (node, w), -1 if absent
    std::vector<int> slot_of;       // [nnode*4] conP slot of (node, class), -1 if absent
    std::vector<int> sslot_of;      // [nnode*4] scale slot
    std::vector<int> scale_list;    // [4*nscale] scale slot per root class and scaled node
    int nslot = 0, nsslot = 0;

    // device buffers
    gb::Item *d_items = nullptr;
    gb::PairDesc *d_pairs = nullptr;
    int *d_label = nullptr, *d_scale_list = nullptr;
    unsigned char *d_z = nullptr;
    unsigned char *d_amb = nullptr;   // unclean data: nChara[256] + CharaMap[256][64] (null: clean)
    double *d_fpatt = nullptr, *d_pi = nullptr, *d_tnode = nullptr;
    gb::DevParams *d_prm = nullptr;
    double *d_Pt = nullptr, *d_conP = nullptr, *d_E = nullptr, *d_scaleF = nullptr;
    double *d_fbar = nullptr, *d_ssum = nullptr, *d_fhK = nullptr, *d_lnf = nullptr, *d_post = nullptr;
    double *d_partial = nullptr, *d_out = nullptr;
    unsigned *d_ticket = nullptr;

    // pinned staging
    gb::DevParams *h_prm = nullptr;
    double *h_tnode = nullptr, *h_out = nullptr;

    // CUDA graphs of the forward evaluation (without / with E messages kept)
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int graph_kernels = 0;
    // BEB: forwards restricted to the items of some site classes (bit c of
    // the mask selects class c), each P(t) then those items level by level
    gb::Item *d_items_cls[16] = {};
    std::vector<int> cls_off[16];
    cudaGraphExec_t graph_cls[16] = {};
    int graph_cls_kernels[16] = {};

    gb::AdjointState *adj = nullptr;
    gb::FastState *fast = nullptr;
    gb::CladeState *clade = nullptr;    // clade models C / D in one evaluation (clade.cu)
    int kernels_last = 0;
    gb::ProfRec *prof = nullptr;
};

namespace gb {
// host staging of one evaluation's parameters into the handle's pinned buffers
int stage_params(gb_handle *h, const Derived *D, const double *blength);
// record one evaluation's device work (copies in, kernels, copies out) on
// h->stream; returns the kernel count or a negative GB_ERR_*
int fp64_record_eval(gb_handle *h, bool grad);
int fast_record_eval(gb_handle *h, bool grad);
int fast_prepare(gb_handle *h, bool grad);     // allocations / kernel attributes before a capture
int fp64_prepare(gb_handle *h, bool grad);
int fast_check_error(gb_handle *h);
// split-precision pieces (fast.cu), each recorded on h->stream; they return
// the number of kernels (copies: 0 or a GB_ERR_*)
int fast_rec_copies_in(gb_handle *h, bool grad);
int fast_rec_pmat(gb_handle *h);      // P (FP64) and its digit planes
int fast_rec_mix(gb_handle *h);       // site-class mixture, lnL
int fast_rec_dmat(gb_handle *h);      // dP/dt terms of the adjoint
int fast_rec_tail(gb_handle *h);      // per-pair and class-weight gradient sums
int fast_rec_copies_out(gb_handle *h, bool grad);
bool fast_persistent(const gb_handle *h);
struct PsliceArgs;
float2 *fast_groot(gb_handle *h);                               // adjoint root seed (nullptr without one)
PsliceArgs fast_pslice_args(gb_handle *h);                      // P digit-plane buffers (batched launches)
void fast_swap_err(gb_handle *h, int *&d_err, int *&h_err);     // exchange the error word (batch staging)
int fast_task_trace(gb_handle *h, int kernel, unsigned long long *out, int cap);
int fast_fault_inject(gb_handle *h, int wait_ms, int withhold);
int persist_task_trace(PersistPlan *pp, int kernel, unsigned long long *out, int cap);
int fast_ns(const gb_handle *h, bool adjoint);
// persistent executors over one or many genes (fast.cu)
void persist_free(PersistPlan *pp);
int persist_build(PersistPlan *pp, gb_handle *const *hs, int n, bool bwd, const Tuning &tune);
int persist_record_fwd(PersistPlan *pp, bool keepE, int ns, cudaStream_t st, gb_handle *prof);
int persist_record_bwd(PersistPlan *pp, int nsb, cudaStream_t st, gb_handle *prof);
// forward pass on the handle's stream (runtime.cu); keepE keeps the edge
// messages for the adjoint
int run_forward(gb_handle *h, const Derived *D, const double *blength, bool keepE, double *neg_lnL,
                double *fhK, double *lnf, gb_stats *stats);
}  // namespace gb
