// Per-gene argument blocks of the kernels that a batch runs as ONE launch over
// all genes (block b works on local block map[b].y of gene map[b].x): P
// assembly, P digit planes, site-class mixture, dP/dt, per-pair gradient
// transform and class-weight sums.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "internal.h"

namespace gb {

struct GradParams;

struct PmatArgs {
    const PairDesc *pairs;
    const int *label;
    const double *tnode;
    const DevParams *prm;
    double *Pt;
    const double *pi;            // codon frequencies (symmetric form of P, see launch_pmat_fp64)
};

struct PsliceArgs {
    const double *Pt64;
    float2 *Pdf;
    __nv_bfloat16 *Bf, *Bb;
};

struct MixArgs {
    const double *fhK, *fpatt;
    const DevParams *prm;
    int npatt, npad, nscale, nblocks;
    double *lnf, *post, *partial;
    unsigned *ticket;
    double *out;
    const double *fbar;          // split precision with a gradient: root sums f~ [4][npad] ...
    float2 *groot;               // ... and the adjoint's root seed fpatt post / f~ as double-float (nullable)
};

struct DmatArgs {
    const DevParams *prm;
    const GradParams *gp;
    double *Dm;
    float2 *UVdf;
};

struct GradHArgs {
    const PairDesc *pairs;
    const int *label;
    const double *tnode;
    const DevParams *prm;
    const float2 *Gpart;
    int nchunk;
    const double *Dm;
    const float2 *UVdf;
    double *out;
};

struct FreqArgs {
    const double *fhK, *lnf, *fpatt;
    int npatt, npad, nscale;
    double *part;
};

void launch_pmat_batched(const PmatArgs *args, const int2 *map, int nblocks, cudaStream_t st);
void launch_pslice_batched(const PsliceArgs *args, const int2 *map, int nblocks, int ns, cudaStream_t st);
void launch_mix_batched(const MixArgs *args, const int2 *map, int nblocks, cudaStream_t st);
void launch_dmat_batched(const DmatArgs *args, const int2 *map, int nblocks, cudaStream_t st);
void launch_gradH_batched(const GradHArgs *args, const int2 *map, int nblocks, cudaStream_t st);
void launch_freq_batched(const FreqArgs *args, const int2 *map, int nblocks, cudaStream_t st);

}  // namespace gb
