/*
 * gbcodeml_codeml.h -- the entry points codeml.c itself calls on its CUDA path,
 * provided by cucodeml_gb300/csrc/codeml_adapter.c, which is compiled into
 * codeml (against codeml's own paml.h / codeml.h) and links libgbcodeml.so.
 *
 *   CUDA_Init                      replaces cuda-codeml.cu:1106 (called at
 *                                  codeml.c:684): creates the library handle from
 *                                  codeml's globals (tree, com.z, com.fpatt,
 *                                  com.pi, com.nodeScale).
 *   CUDA_ScheduleConditionalPNode  replaces cuda-codeml.cu:1336 (called per site
 *                                  class from CUDA_fx_r, treesub.c:7583): the
 *                                  first class of an evaluation runs all four
 *                                  classes on the GPU from codeml's _UU/_VV/_Root,
 *                                  Qfactor_NS_branch and com.freqK; every call
 *                                  copies its class into com.fhK + ir*npatt.
 *                                  Clade models C/D (model = 3, two branch
 *                                  types): their three classes in one
 *                                  evaluation from _UU/_VV/_Root[0..3]
 *                                  (gb_eval_clade_uvr).
 *   CUDA_FreeAll                   replaces cuda-codeml.cu:1162 (codeml.c:695).
 *   GB_dfun                        new: ming2's gradient hook
 *                                  (tools.c:6361-6363, `dfun`), the analytic
 *                                  gradient of -lnL in codeml's x space
 *                                  (branch-site models A and B, clade models
 *                                  C and D); pass it instead of NULL at
 *                                  codeml.c:688.
 *   GB_BEB                         new: the Bayes empirical Bayes analysis of
 *                                  models A and B (and of the clade models C
 *                                  and D: postSite[3*npatt], grid = the
 *                                  postpara rows p0, p1 (-1), w0, [w1], w2,
 *                                  w3) on the GPU at codeml's final
 *                                  x (kappa and branch lengths; the Qfactors
 *                                  are codeml's Qfactor_NS_branch, as its BEB
 *                                  reads them): fills
 *                                  lfunNSsites_ACD's postSite[4*npatt], the w0
 *                                  and w2 rows of its postpara (grid[20..39]),
 *                                  postp0p1[100] and log f(X), S1, S2
 *                                  (lnfX[3]); replaces codeml.c:6697-6775 for
 *                                  model A.  Makes its own handle, since
 *                                  CUDA_FreeAll has run by then.
 *   GB_HessianSKT2004              new: HessianSKT2004 (treesub.c:6979-7048)
 *                                  with the same arguments and results (g and
 *                                  H at codeml's x, H before codeml negates
 *                                  it), its 2 np likelihood evaluations on the
 *                                  GPU; call it in place of HessianSKT2004 at
 *                                  codeml.c:764 for getSE = 1 (branch-site
 *                                  models A and B).
 *
 * CUDA_lfundG and CUDA_fx_r stay codeml's own (treesub.c:7397, 7554).  On any
 * library error these functions print the library's message and exit(-1), as
 * the reference's cutilSafeCall does (cuda-codeml.cu:20-39); the C ABI below
 * them returns status codes instead.
 */
#ifndef GBCODEML_CODEML_H
#define GBCODEML_CODEML_H

#ifdef __cplusplus
extern "C" {
#endif

void CUDA_Init(double *x);
void CUDA_ScheduleConditionalPNode(int ir, int ig, double *x);
void CUDA_FreeAll(void);
int GB_dfun(double x[], double *f, double dx[], int n);
int GB_BEB(double x[], int np, double postSite[], double grid[], double p0p1[], double lnfX[]);
int GB_HessianSKT2004(double xmle[], double lnLm, double g[], double H[]);

#ifdef __cplusplus
}
#endif

#endif /* GBCODEML_CODEML_H */
