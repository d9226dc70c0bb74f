// Types shared by the split-precision kernels (k_fast.cu, k_fast_bwd.cu) and
// their host code (fast.cu).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "internal.h"
#include "adjoint_internal.h"

namespace gb {

constexpr int FAST_MT = 128;   // patterns per CTA tile in the split-precision kernels

// one unit of work of a persistent kernel: (gene, item, tile); for dlnL/dP
// item = pair and tile = pattern chunk
struct Task {
    int gene, item, tile;
    int edge;        // adjoint: the one child edge of the item this task handles (-1: all of them)
};

// control words of a persistent executor (device memory): the evaluation
// epoch (ready flags hold the epoch of the evaluation that wrote them) and
// the task counters of the three persistent kernels
// CTL_SKEW, CTL_WAIT_MS: the bounded flag waits compare against epoch + skew
// (0: the current evaluation; gb_fault_inject sets 1, a value nothing writes)
// and give up after CTL_WAIT_MS milliseconds (0: 2000)
enum { CTL_EPOCH = 0, CTL_FWD = 1, CTL_BWD = 2, CTL_GRADP = 3, CTL_SKEW = 4, CTL_WAIT_MS = 5, CTL_WORDS = 6 };

struct FastFwdArgs;
struct FastBwdArgs;

// the persistent launches of one executor (a handle, or a batch of genes):
// per-gene argument blocks, task lists and control words, all in device memory
struct PersistPlan {
    unsigned *ctl = nullptr;                         // [CTL_WORDS]
    FastFwdArgs *d_fargs[2] = {nullptr, nullptr};    // per gene, without / with edge messages
    FastBwdArgs *d_bargs = nullptr;                  // per gene
    Task *d_ftask = nullptr, *d_btask = nullptr, *d_gtask = nullptr;
    int nftask = 0, nbtask = 0, ngtask = 0;
    int nblock = 0;                                  // CTAs per persistent launch (one per SM)
    int ngene = 0;
    bool has_bwd = false;
    unsigned long long *trace[3] = {nullptr, nullptr, nullptr};   // per kernel, when tracing
    bool tracing = false;
};

struct FastFwdArgs {
    const Item *items;
    int npad;
    const unsigned char *z;
    const double *Pt64;          // FP64 P (input of pslice)
    const float2 *Pdf;           // [npair][64][64] Pt as double-float
    const __nv_bfloat16 *Bf;     // [npair][NS][64][64] digit planes of P (forward)
    __nv_bfloat16 *Bb;           // [npair][NS][64][64] digit planes of Pt (adjoint)
    float2 *conP;                // [nslot][npad][64] normalised conditional likelihoods
    int *expo;                   // [nslot][npad] their power-of-two exponents
    float2 *E;                   // [nslot*3][npad][64] edge messages (nullable)
    const double *pi;
    double *fbar, *ssum, *fhK;   // [4][npad]
    int *expo_root;              // [4][npad]
    int *err;                    // set to 1 by a CTA whose bounded wait gave up
    unsigned *ready;             // [nslot][ntile] epoch of the last write of (slot, tile)
    int ntile;
};

struct FastBwdArgs {
    const BItem *bitems;
    int npad, npatt, nchunk;
    const float2 *E;             // forward edge messages
    const float2 *conP;          // forward normalised conditional likelihoods
    const int *expo, *expo_root;
    const __nv_bfloat16 *Bb;     // digit planes of Pt
    float2 *Ebar;                // [nslot*3][npad][64] normalised dlnL/dE
    int *ebexp;                  // [nslot*3][npad]
    float2 *Abar;                // [nslot][npad][64] normalised dlnL/dL~
    int *aexp;                   // [nslot][npad]
    const double *fpatt, *post, *fbar, *pi;
    const Contrib *contrib;
    const int *coff;
    const unsigned char *z;
    float2 *Gpart;               // [npair][nchunk][64][64] dlnL/dP partials, double-float
    int *err;
    int nsP;                     // digit planes stored per pair in Bb
    int gchunk;                  // patterns per dlnL/dP partial
    unsigned *ready;             // [nslot][ntile] epoch of the last Abar write of (slot, tile)
    int ntile;
    const float2 *Pdf;           // P as double-float (a tip's edge message is a row of it)
    const float2 *groot;         // [4][npad] root seed fpatt post / f~ (double-float)
    const float2 *pidf;          // [64] codon frequencies (double-float, zero padded)
};

cudaError_t init_fast_kernels(int ns);
cudaError_t init_fast_bwd_kernels(int ns);
cudaError_t init_umma_kernels(int ns);
void launch_prune_umma(const FastFwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st);
void launch_bwd_umma(const FastBwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st);
void launch_gradP_umma(const FastBwdArgs &a, int ns, int npair, cudaStream_t st);
void launch_bwd_fast(const FastBwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st);
void launch_gradP_fast(const FastBwdArgs &a, int ns, int npair, cudaStream_t st);
void launch_pslice(const FastFwdArgs &a, int ns, int npair, bool cm, cudaStream_t st);
void launch_prune_fast(const FastFwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st);
void launch_bump(unsigned *ctl, cudaStream_t st);
// trace: nullable, TRACE_WORDS per task (claim ns, dependencies met ns, four
// phase stamps, end ns, SM); gb_task_trace returns TRACE_OUT words per task
constexpr int TRACE_WORDS = 8;
constexpr int TRACE_OUT = 4 + TRACE_WORDS;
void launch_prune_persist(const FastFwdArgs *genes, const Task *tasks, int ntask, unsigned *ctl, int ns,
                          int nblock, unsigned long long *trace, cudaStream_t st);
void launch_bwd_persist(const FastBwdArgs *genes, const Task *tasks, int ntask, unsigned *ctl, int ns,
                        int nblock, unsigned long long *trace, cudaStream_t st);
void launch_gradP_persist(const FastBwdArgs *genes, const Task *tasks, int ntask, unsigned *ctl, int ns,
                          int nblock, unsigned long long *trace, cudaStream_t st);

}  // namespace gb
