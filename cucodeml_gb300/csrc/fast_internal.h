// Types shared by the split-precision kernels (k_fast.cu, k_fast_bwd.cu) and
// their host code (fast.cu).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "internal.h"
#include "adjoint_internal.h"

namespace gb {

constexpr int FAST_MT = 128;   // patterns per CTA tile in the split-precision kernels

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
    double *Gpart;               // [npair][nchunk][64][64]
    int *err;
    int nsP;                     // digit planes stored per pair in Bb
    int gchunk;                  // patterns per dlnL/dP partial
};

cudaError_t init_fast_kernels(int ns);
cudaError_t init_fast_bwd_kernels(int ns);
cudaError_t init_umma_kernels(int ns);
void launch_prune_umma(const FastFwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st);
void launch_bwd_umma(const FastBwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st);
void launch_gradP_umma(const FastBwdArgs &a, int ns, int npair, cudaStream_t st);
void launch_bwd_fast(const FastBwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st);
void launch_gradP_fast(const FastBwdArgs &a, int ns, int npair, cudaStream_t st);
void launch_pslice(const FastFwdArgs &a, int ns, int npair, cudaStream_t st);
void launch_prune_fast(const FastFwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st);

}  // namespace gb
