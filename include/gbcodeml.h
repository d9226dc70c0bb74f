/*
 * gbcodeml.h -- C ABI of libgbcodeml.so, a GB300 (sm_103a) implementation of
 * PAML codeml's branch-site model A likelihood hot path (and, on the same
 * kernels, model B, the clade models C / D and the site models).
 *
 * Everything here is plain C: pointers, sizes and status codes.  No call
 * exits the process; every entry point returns GB_OK (0) or a negative
 * GB_ERR_* code, and gb_last_error() gives a one-line reason.
 *
 * What each entry point replaces in the reference (paths relative to the
 * reference project):
 *
 *   gb_create / gb_destroy   CUDA_Init / CUDA_FreeAll (cuda-codeml.cu:1106-1124,
 *                            1162-1181) -- device set-up per tree and data set,
 *                            but with all inputs passed explicitly instead of
 *                            being read from codeml's globals (codeml.h:67-105).
 *   gb_eval_uvr              CUDA_fx_r + CUDA_lfundG (treesub.c:7397-7450,
 *                            7554-7595): P(t) for every branch from the host's
 *                            U, V, Root (codeml's _UU/_VV/_Root, eigenQcodon
 *                            codeml.c:2516-2520), pruning over the 4 site classes,
 *                            node scaling, and the site-class mixture; fills
 *                            fhK[4*npatt] exactly as CUDA_fx_r fills com.fhK and
 *                            returns -lnL as CUDA_lfundG does.
 *   gb_eval                  the same from the natural model-A parameters
 *                            (branch lengths, kappa, w0, w2, p0, p1): the library
 *                            builds Q, its eigen solution and the Qfactors
 *                            (SetParametersNSsites codeml.c:2488-2521) itself.
 *                            Optionally returns the analytic gradient of -lnL
 *                            (the reference has none: ming2's dfun hook,
 *                            tools.c:6361-6363, is passed NULL at codeml.c:688
 *                            and gradientB tools.c:6326-6350 differentiates
 *                            numerically).
 *   gb_dfun_x                ming2's dfun signature (tools.c:6361-6363) over
 *                            codeml's parameter vector x (branch lengths in
 *                            codeml's branch order, kappa, p0/p1 in codeml's
 *                            transformed or untransformed form, w0, w2).
 *   gb_patterns              PatternWeight + EncodeSeqs (treesub.c:1075-1143,
 *                            1302-1439) and F3x4 codon frequencies
 *                            (codeml.c:3475-3570, 3732-3742) for clean codon data.
 *   gb_neb                   the NEB site-class posteriors codeml prints
 *                            (lfunNSsites_rate codeml.c:5079-5129).
 *   gb_ng86                  DistanceMatNG86 (treesub.c:2270-2366): pairwise
 *                            Nei-Gojobori dS, dN from per-codon-pair tables.
 *   gb_se_opg / gb_hessian_x standard errors: codeml's getSE = 1 Hessian
 *                            approximation HessianSKT2004 (treesub.c:6979-7048)
 *                            with its 2 np evaluations on the device; and the
 *                            Hessian from differences of the analytic gradient.
 *   gb_beb                   the Bayes empirical Bayes site analysis of model A,
 *                            lfunNSsites_ACD (codeml.c:6617-6826): 121 full
 *                            prunings over an omega grid and the integration
 *                            over a 10^4-point parameter grid, on the device.
 *   gb_eval_b                branch-site model B (NSsites = 3, codeml.c:
 *                            2427-2436): model A with a free w1, with gradient.
 *   gb_eval_clade_uvr /      clade models C and D with two branch types
 *   gb_eval_clade /          (model = 3, codeml.c:2437-2446, 2522-2539) in one
 *   gb_dfun_clade_x /        evaluation, from codeml's four eigen solutions or
 *   gb_neb_clade             the library's own set-up; gradient, ming2's dfun
 *                            and the NEB posteriors.
 *   gb_beb_tables /          f(x_h | w) on other omega grids and the clade-C /
 *   gb_beb_clade             clade-D BEB grid integrals (10^5 / 10^6 points).
 *   gb_beta_classes          M7 / M8's discretised beta (DiscreteNSsites
 *                            codeml.c:2728-2770).
 *   gb_batch_*               many alignments in one graph launch per
 *                            evaluation (models A and B).
 *
 * The five symbols codeml.c itself calls (CUDA_Init, CUDA_lfundG, CUDA_fx_r,
 * CUDA_ScheduleConditionalPNode, CUDA_FreeAll; codeml.h:67-85) are provided
 * by the adapter cucodeml_gb300/csrc/codeml_adapter.c, declared in
 * gbcodeml_codeml.h, which is compiled into codeml against its own headers.
 *
 * Threading: one handle per host thread; calls on one handle are not
 * re-entrant.  The library owns device memory; the caller owns every host
 * array passed in or out.
 */
#ifndef GBCODEML_H
#define GBCODEML_H

#ifdef __cplusplus
extern "C" {
#endif

#define GB_OK            0
#define GB_ERR_ARG      -1   /* malformed tree / data / sizes */
#define GB_ERR_CUDA     -2   /* CUDA runtime error (message in gb_last_error) */
#define GB_ERR_OOM      -3   /* device or host allocation failed */
#define GB_ERR_PARAM    -4   /* parameter values outside the model (p0+p1 ~ 0, t < 0, ...) */
#define GB_ERR_TIMEOUT  -5   /* a bounded device-side wait gave up */
#define GB_ERR_STATE    -6   /* call on a destroyed / unfinished handle */
#define GB_ERR_NODEVICE -7   /* no CUDA device */

#define GB_NCODE 61           /* universal code, sense codons */

/* precision of the pruning contraction */
#define GB_PREC_FP64     0    /* FP64 throughout: the drop-in (<=1e-9 relative lnL) */
#define GB_PREC_FAST     1    /* split precision: each operand cut into 7-bit digit planes
                                 held exactly in bf16, digit products summed exactly in FP32
                                 on the tensor cores, levels combined in double-float; P(t),
                                 the root sum, logs and the lnL sum stay FP64 */
#define GB_PREC_FAST_NS(n) (16 + (n))  /* GB_PREC_FAST with n = 5..8 digit planes (default 8) */

typedef struct gb_handle gb_handle;

typedef struct {
    int ns;                       /* taxa; tips are nodes 0..ns-1 */
    int nnode;                    /* nodes incl. root (2ns-2 for an unrooted binary tree) */
    int root;                     /* root node id (>= ns) */
    const int *father;            /* [nnode] father id, -1 for the root */
    const int *label;             /* [nnode] branch label: 0 background, 1 foreground (#1) */
    int npatt;                    /* site patterns */
    const unsigned char *z;       /* [ns*npatt] sense codon 0..60 per tip and pattern */
    const double *fpatt;          /* [npatt] pattern counts */
    const double *pi;             /* [61] codon frequencies */
    const char *node_scale;       /* [nnode] 1 = scale conditional likelihoods at this node
                                     (codeml's com.nodeScale); NULL = codeml's own rule
                                     (SetNodeScale, treesub.c:6917-6937) */
    int precision;                /* GB_PREC_* */
    int device;                   /* CUDA device ordinal */
} gb_problem;

typedef struct {
    const double *blength;        /* [nnode] length of the branch above each node (root ignored) */
    double kappa, omega0, omega2; /* omega1 is 1 */
    double p0, p1;                /* untransformed proportions, p0 + p1 < 1 */
} gb_params;

typedef struct {
    double *d_blength;            /* [nnode] d(-lnL)/d(branch length above node); root entry 0 */
    double d_kappa, d_omega0, d_omega2, d_p0, d_p1;
} gb_grad;

typedef struct {
    double ms_host;               /* host time in the call (set-up, copies, waits) */
    double ms_device;             /* device time of the evaluation (CUDA events) */
    int kernels;                  /* kernel launches made by the call */
    int nscale;                   /* scaled nodes */
    double h2d_bytes;             /* bytes copied host -> device by the call */
    double d2h_bytes;             /* bytes copied device -> host by the call */
} gb_stats;

/* kernel classes reported by gb_profile */
#define GB_K_PMAT     0           /* P(t) assembly */
#define GB_K_PRUNE    1           /* pruning levels (forward contraction) */
#define GB_K_MIX      2           /* site-class mixture, log, sum */
#define GB_K_BWD      3           /* adjoint levels (backward contraction) */
#define GB_K_GRADP    4           /* dlnL/dP accumulation over patterns */
#define GB_K_GRADH    5           /* eigen-basis contraction to parameter derivatives */
#define GB_K_OTHER    6           /* small set-up / reduction kernels */
#define GB_NKCLASS    7

/* Library version string. */
const char *gb_version(void);

/* One-line description of the last error on this thread. */
const char *gb_last_error(void);

/* Create a handle for one tree and data set; uploads everything that does not
   change between evaluations.  Replaces CUDA_Init (cuda-codeml.cu:1106). */
int gb_create(const gb_problem *prob, gb_handle **out);

/* gb_create for data with gaps and ambiguous codons (codeml's cleandata = 0):
   z may hold codes >= 61, each standing for the nchara[z] sense codons
   charamap[64 * z + 0 .. nchara[z] - 1] (codeml's nChara[256] and
   CharaMap[256][64] from SetMapAmbiguity treesub.c:1146-1200, as
   EncodeSeqs treesub.c:1075-1143 numbers them).  A tip with such a code
   contributes the sum of its transition probabilities over those codons, as
   the reference's unclean tip kernels (cuda-codeml.cu:166-204) and
   ConditionalPNode (codeml.c:3438-3445) do.  GB_PREC_FP64 only; the forward
   evaluation, the adjoint gradient, BEB, NEB and standard errors all take
   such data.  GB_ERR_ARG for a code that stands for no sense codon. */
int gb_create_unclean(const gb_problem *prob, const unsigned char *nchara, const unsigned char *charamap,
                      gb_handle **out);

/* Free device memory and the handle.  Replaces CUDA_FreeAll (cuda-codeml.cu:1162). */
int gb_destroy(gb_handle *h);

/* Number of scaled nodes the handle uses (codeml's com.NnodeScale). */
int gb_nscale(const gb_handle *h);

/*
 * Evaluate from the host's eigen solutions, as codeml's CUDA_lfundG does.
 *   U[i], V[i]: 61x61 row-major (Q_i = U diag(Root_i) V), Root[i]: 61, for
 *   i = 0,1,2 the w0, w1 = 1, w2 matrices (codeml's _UU/_VV/_Root);
 *   qfactor[2]: Qfactor_NS_branch for background / foreground branches;
 *   freqK[4]: site-class proportions; blength[nnode]: branch lengths.
 * Outputs (each may be NULL): *neg_lnL; fhK[4*npatt] as codeml's com.fhK
 * (log f + scale logs when any node is scaled, else f); lnf[npatt] per-pattern
 * log f as codeml writes to its lnf file.
 */
int gb_eval_uvr(gb_handle *h, const double *const U[3], const double *const V[3],
                const double *const Root[3], const double qfactor[2], const double freqK[4],
                const double *blength, double *neg_lnL, double *fhK, double *lnf,
                gb_stats *stats);

/*
 * Clade models C and D with two branch types (codeml model = 3, NSsites = 2
 * or 3, ncatG = 3) in one evaluation: the eigen solutions of w0, w1, w2
 * (branch type 0's third class) and w3 (branch type 1's) as codeml's
 * _UU/_VV/_Root[0..3], the two branch types' Qfactors and the three class
 * weights (SetParametersNSsites codeml.c:2437-2446, 2522-2539;
 * Set_UVR_BranchSite codeml.c:2545-2568).  Branch labels 0 / 1 of gb_problem
 * are the branch types.  fhK (may be NULL) receives codeml's fhK of the three
 * classes [3][npatt]; -lnL is codeml's mixture of them (lfundG).  Replaces the
 * clade route of CUDA_ScheduleConditionalPNode (CUDA_fx_r treesub.c:7554-7595
 * with com.model = 3).  FP64 handles; the first call builds the three-class
 * schedule (its own conditional likelihoods and transition matrices).
 */
int gb_eval_clade_uvr(gb_handle *h, const double *const U[4], const double *const V[4],
                      const double *const Root[4], const double qfactor[2], const double freqK[3],
                      const double *blength, double *neg_lnL, double *fhK, double *lnf,
                      gb_stats *stats);

/* gb_eval_clade_uvr from the clade model's parameters, set up by the
   library: kappa, the class weights p0, p1 (p2 = 1 - p0 - p1) and omega[4] =
   (w0, w1, w2, w3) -- w1 = 1 under clade model C, free under D; w2 is the
   third class's omega on branch type 0, w3 on branch type 1 (codeml.c:
   2522-2539).  blength in node order.  grad (may be NULL): the analytic
   gradient of -lnL, [nnode] by branch length (node order, 0 at the root) then
   kappa, p0, p1, w0, w1, w2, w3 (the adjoint of the FP64 path).  FP64 handles. */
int gb_eval_clade(gb_handle *h, const double *blength, double kappa, double p0, double p1,
                  const double omega[4], double *neg_lnL, double *grad, double *fhK, double *lnf,
                  gb_stats *stats);

/* codeml's naive empirical Bayes (NEB) site-class posteriors under the
   clade models (lfunNSsites_rate codeml.c:5079-5129) at gb_eval_clade's
   parameters: post [3][npatt] (pattern order), -lnL in *neg_lnL (may be
   NULL).  FP64 handles. */
int gb_neb_clade(gb_handle *h, const double *blength, double kappa, double p0, double p1,
                 const double omega[4], double *post, double *neg_lnL);

/* gb_eval_clade in codeml's x space for ming2's dfun under clade models:
   x = branch lengths (bnode[i] = node of x[i]), kappa, p0, p1 (codeml's
   transformed proportions unless lastround), w0, [w1 when model_d], w2, w3;
   n = nbranch + 6 (clade C) or + 7 (clade D).  f = -lnL, dx = its gradient. */
int gb_dfun_clade_x(gb_handle *h, const int *bnode, int lastround, int model_d, const double *x, int n,
                    double *f, double *dx);

/*
 * Evaluate -lnL from natural parameters; if grad != NULL also the analytic
 * gradient of -lnL (adjoint sweep).  fhK / lnf / stats may be NULL.
 */
int gb_eval(gb_handle *h, const gb_params *prm, double *neg_lnL, gb_grad *grad,
            double *fhK, double *lnf, gb_stats *stats);

/* gb_eval for branch-site model B (codeml NSsites = 3, ncatG = 3), whose
   site class 1 has a free omega1 where model A fixes it at 1: the second
   eigen solution is Q(kappa, omega1) and omega1 enters both branch types'
   mean rates behind the Qfactors (SetParametersNSsites codeml.c:2427-2436,
   2488-2521); classes, their omega map and the pruning are model A's.  Any
   precision.  With grad, *d_omega1 (may be NULL) receives d(-lnL)/d omega1
   beside the other derivatives.  gb_dfun_x takes model B's x (branch lengths,
   kappa, p0, p1, w0, w1, w2) when n = nbranch + 6. */
int gb_eval_b(gb_handle *h, const gb_params *prm, double omega1, double *neg_lnL, gb_grad *grad,
              double *d_omega1, double *fhK, double *lnf, gb_stats *stats);

/*
 * Bayes empirical Bayes (BEB) analysis of branch-site model A at prm
 * (normally the MLE), as codeml's lfunNSsites_ACD (codeml.c:6617-6826, with
 * get_grid_para_like_ACD 6419-6530, get_pclassM_iw_ACD 6532-6615 and the BEB
 * branch of GetPMatBranch treesub.c:7289-7301) computes it after the
 * optimisation.  kappa, the branch lengths and the branch Qfactors stay at
 * prm; omega runs over a grid of GB_BEB_GRID values of w0 in (0, 1) and of w2
 * in (1, 11), and (p0, p1) over GB_BEB_GRID^2 triangles of the ternary plot.
 * f(x_h | w) is computed for the GB_BEB_OMEGA_SETS omega sets
 *   [0, 10)        background = foreground = w0_i        (class 0)
 *   10             background = foreground = 1           (class 1)
 *   11 + 10 i + j  background w0_i, foreground w2_j      (class 2a)
 *   111 + j        background 1, foreground w2_j         (class 2b)
 * by full FP64 prunings on the device (sets sharing a background omega
 * recompute only the foreground branch's path to the root); the grid
 * integration runs on the device too.
 * Outputs (each may be NULL):
 *   lnfw[121*npatt]  log f(x_h | omega set) (log f + scale logs)
 *   post[4*npatt]    posterior of site classes 0, 1, 2a, 2b per pattern
 *                    (codeml's rst "BEB probabilities"; P(w>1) = 2a + 2b)
 *   grid[4*10]       posterior of the grid values of p0, p1 (rows of -1, as
 *                    codeml prints them), w0 and w2 ("Posterior on the grid")
 *   p0p1[100]        posterior over the (p0, p1) triangles
 *   lnfX[3]          log f(X) as codeml prints it, and its scale terms S1, S2
 * Needs a GB_PREC_FP64 handle (GB_ERR_STATE otherwise).
 */
#define GB_BEB_GRID        10
#define GB_BEB_OMEGA_SETS  121
int gb_beb(gb_handle *h, const gb_params *prm, double *lnfw, double *post, double *grid,
           double *p0p1, double *lnfX, gb_stats *stats);

/*
 * gb_beb with the two branch Qfactors given (codeml's Qfactor_NS_branch,
 * which its BEB reads at the MLE, GetPMatBranch treesub.c:7289-7301) instead
 * of derived from model A's parameters: the same analysis for branch-site
 * model B, whose Qfactors involve its free w1 (codeml runs model A's BEB grid
 * for it).  blength[nnode]: branch lengths by node.  wmean[npatt], wsd[npatt]
 * (each may be NULL): the posterior mean and standard deviation of the site's
 * w, taking w0_i, 1 and w2_j as the w of classes 0, 1 and 2a/2b -- on a tree
 * with every branch in the foreground, the "post mean +- SE for w" codeml
 * prints for M2a (lfunNSsites_M2M8 codeml.c:6331-6374).
 */
int gb_beb_qf(gb_handle *h, const double *blength, double kappa, const double qfactor[2], double *lnfw,
              double *post, double *grid, double *p0p1, double *lnfX, double *wmean, double *wsd,
              gb_stats *stats);

/*
 * The 121 log f(x_h | w) tables of gb_beb_qf (lnfw[121*npatt], same set
 * order) with other omega grids: w_slot0[10] in place of the w0 grid and
 * w_slot2[10] in place of the w2 grid; no grid integration.  Serves BEB
 * analyses on other grids, e.g. codeml's clade model C (w2, w3 in (0, 3),
 * lfunNSsites_ACD codeml.c:6617-6826 with modelACD = mC): its third class's
 * sets (w2_i background, w3_j foreground) are sets 11 + 10 i + j here.
 */
int gb_beb_tables(gb_handle *h, const double *blength, double kappa, const double qfactor[2],
                  const double w_slot0[GB_BEB_GRID], const double w_slot2[GB_BEB_GRID], double *lnfw,
                  gb_stats *stats);

/*
 * The grid integral of codeml's BEB under the clade models with two branch
 * types (lfunNSsites_ACD codeml.c:6617-6826, modelACD = mC / mD), on the
 * device, from host tables lnfw [nsets][npatt] of log f(x_h | w):
 *   model_d = 0 (clade C): 111 sets -- 0..9 w0 (grid in (0, 1)) on every
 *     branch, 10 w = 1 on every branch, 11 + 10 i + j w2_i background and
 *     w3_j foreground (grids in (0, 3)); 10^5 grid points;
 *   model_d = 1 (clade D): 120 sets -- 0..9 w0 (grid in (0, 0.5)), 10..19 w1
 *     (grid in (0.5, 1.5)) on every branch, 20 + 10 i + j as above; 10^6
 *     grid points.
 * (gb_beb_tables computes such tables with its two eigen slots on these
 * grids.)  Outputs (each may be NULL): post [3*npatt] site-class posteriors,
 * grid [4*10] posterior on the w0, w1 (-1 under C), w2 and w3 grids, p0p1
 * [100] posterior of the (p0, p1) triangles, lnfX [3] = log f(X) as codeml
 * prints it, S1, S2.  No counterpart in the reference's GPU code (codeml
 * integrates on one CPU core).
 */
int gb_beb_clade(gb_handle *h, int model_d, const double *lnfw, double *post, double *grid, double *p0p1,
                 double *lnfX, gb_stats *stats);

/* The whole clade-C / clade-D BEB at the MLE: the log f tables of
   gb_beb_clade from gb_beb_tables on the clade grids (branch lengths in
   node order, kappa and the branch types' Qfactors as codeml's
   lfunNSsites_ACD reads them), then gb_beb_clade; outputs as there. */
int gb_beb_clade_bl(gb_handle *h, int model_d, const double *blength, double kappa, const double qfactor[2],
                    double *post, double *grid, double *p0p1, double *lnfX, gb_stats *stats);

/*
 * Naive empirical Bayes (NEB) posteriors of the four site classes at prm, as
 * codeml's lfunNSsites_rate prints them ("Naive Empirical Bayes (NEB)
 * probabilities", codeml.c:5079-5129): post[c*npatt + h] = freqK_c f_c(h) /
 * sum_k freqK_k f_k(h), from the mixture of one FP64 evaluation; *neg_lnL
 * (may be NULL) its -lnL.  Needs a GB_PREC_FP64 handle.
 */
int gb_neb(gb_handle *h, const gb_params *prm, double *post, double *neg_lnL);

/*
 * Standard errors as codeml computes them with getSE = 1 (codeml.c:754-783):
 * the Hessian approximation of HessianSKT2004 (treesub.c:6979-7048),
 *   H = -sum_h fpatt_h s_h s_h^T,  s_h,i = (log f_h(x + e_i eh_i)
 *       - log f_h(x - e_i eh_i)) / (2 eh_i),  eh_i = 2 small_diff (|x_i| + 1),
 * and SE_i = sqrt([(-H)^-1]_ii), -1 where that is not positive.
 *   x[n]: codeml's parameter vector as Forestry leaves it after the fit
 *         (codeml.c:713-729): branch lengths by branch index (bnode[ib] is the
 *         node of branch ib), kappa, p0, p1, w0, w2 (p0, p1 untransformed);
 *         n = nnode - 1 + 5; branch-site model B: ..., w0, w1, w2 with
 *         n = nnode - 1 + 6.  small_diff: codeml's Small_Diff.
 * Outputs (each may be NULL): g[n] = dlnL/dx from the same 2n evaluations,
 * H[n*n] (before codeml negates it), se[n].  The 2n FP64 evaluations run on
 * the device back to back.  Needs a GB_PREC_FP64 handle.  Returns
 * GB_ERR_PARAM (se all -1) when -H is singular.
 */
int gb_se_opg(gb_handle *h, const int *bnode, const double *x, int n, double small_diff, double *g,
              double *H, double *se, gb_stats *stats);

/* gb_se_opg under the clade models C (model_d = 0) and D: x = branch
   lengths (bnode as there), kappa, p0, p1 (untransformed), w0, [w1 under D],
   w2, w3; n = nnode - 1 + 6 (C) or + 7 (D).  The 2n evaluations are
   gb_eval_clade calls.  FP64 handles. */
int gb_se_opg_clade(gb_handle *h, const int *bnode, int model_d, const double *x, int n, double small_diff,
                    double *g, double *H, double *se);

/*
 * The Hessian of -lnL over codeml's x (the layout and p0/p1 convention of
 * gb_dfun_x) by central differences of the analytic gradient, step
 * rel_step (|x_i| + 1) (rel_step <= 0: 1e-5), symmetrised: 2n gradient
 * evaluations in place of the 2n^2 likelihood evaluations of codeml's
 * Hessian (tools.c:5774-5810).  se (may be NULL): sqrt of the diagonal of
 * H^-1 (-1 where not positive).  Any precision.
 */
int gb_hessian_x(gb_handle *h, const int *bnode, int lastround, const double *x, int n, double rel_step,
                 double *H, double *se);

/*
 * ming2-compatible gradient hook over codeml's parameter vector
 * x = [branch lengths by branch index (bnode[ib] is the node of branch ib),
 *      kappa, p0', p1', w0, w2]; p' are codeml's f_and_x transforms
 * (tools.c:1280-1305) unless lastround != 0, then p0, p1 themselves.
 * Writes f = -lnL and dx = d(-lnL)/dx.  n must be nnode-1+5.
 */
int gb_dfun_x(gb_handle *h, const int *bnode, int lastround, const double *x, int n,
              double *f, double *dx);

/*
 * Pattern compression of a clean codon alignment.
 *   codons[ns*ncodon]: sense codon id 0..60 per species (row) and site.
 * Outputs: *npatt; z[ns*ncodon] (first ns*npatt entries used, row stride
 * npatt); fpatt[ncodon] (first npatt used); pi[61] F3x4 frequencies.
 * Pattern order and counts are those codeml produces.
 */
int gb_patterns(int ns, int ncodon, const int *codons, int *npatt, unsigned char *z,
                double *fpatt, double *pi);

/*
 * Pairwise Nei-Gojobori (1986) distances of a clean codon alignment, as
 * codeml prints them before the fit (DistanceMatNG86 treesub.c:2270-2366,
 * difcodonNG tools.c:305-420).  Host only (no device).
 *   z[ns*npatt], fpatt[npatt]: patterns as from gb_patterns.
 * Outputs [ns*ns], symmetric, zero diagonal: dS and dN (-1 where NG86 does not
 * apply, as codeml prints them); dist (may be NULL): codeml's SeqDistance,
 * (S dS + N dN) 3 / (S + N) with inapplicable distances set to 3.
 * codeml prints dN/dS as dN / dS where both are positive, else -1.
 */
int gb_ng86(int ns, int npatt, const unsigned char *z, const double *fpatt, double *dS, double *dN,
            double *dist);

/*
 * Batched evaluation of many independent alignments ("genes"), each with its
 * own tree, patterns, codon frequencies and parameters (one device, one
 * precision for the whole batch).  gb_batch_eval evaluates every gene
 * (-lnL, and gradients when grads != NULL) with one CUDA-graph launch in
 * which each gene's work is an independent branch; the host model set-up
 * runs on all host cores.  prm, neg_lnL and grads are arrays of ngene.
 * gb_batch_replay: as gb_replay, for the whole batch.
 */
typedef struct gb_batch gb_batch;
int gb_batch_create(int ngene, const gb_problem *probs, gb_batch **out);
int gb_batch_size(const gb_batch *b);
int gb_batch_eval(gb_batch *b, const gb_params *prm, double *neg_lnL, gb_grad *grads, gb_stats *stats);
/*
 * gb_batch_eval in two halves, so that the host work of one batch overlaps
 * the device work of another: gb_batch_submit runs the host model set-up
 * and launches the batch's graph without waiting for it (after `after`'s
 * last submitted graph when after != NULL, so that the device runs the two
 * back to back); gb_batch_collect waits for it and fills neg_lnL (and grads,
 * if the evaluation was submitted with with_grad).  One evaluation may be
 * outstanding per batch (GB_ERR_STATE otherwise).  Two batches over two
 * halves of a set of genes, submitted alternately, keep the device busy
 * while the host prepares the other half.
 */
int gb_batch_submit(gb_batch *b, const gb_params *prm, int with_grad, const gb_batch *after);
int gb_batch_collect(gb_batch *b, double *neg_lnL, gb_grad *grads, gb_stats *stats);
/* Branch-site model B over a batch (gb_eval_b per gene, codeml NSsites = 3):
   gb_batch_submit with each gene's free omega1[i]; after gb_batch_collect
   of an evaluation submitted with gradient, gb_batch_omega1_grad gives each
   gene's d(-lnL)/d omega1 (the other derivatives are in grads). */
int gb_batch_submit_b(gb_batch *b, const gb_params *prm, const double *omega1, int with_grad,
                      const gb_batch *after);
int gb_batch_omega1_grad(const gb_batch *b, double *d_omega1);
int gb_batch_replay(gb_batch *b, int iters, int with_grad, double *ms);
int gb_batch_destroy(gb_batch *b);

/*
 * Measurement hooks (used by the benchmark):
 *   gb_replay   re-runs the device work of the last gb_eval on this handle
 *               `iters` times with its inputs resident on the device (no host
 *               work, no copies) and returns the device time in *ms (CUDA
 *               events on the handle's stream).  with_grad selects the
 *               lnL+gradient work; it requires a previous gb_eval with grad.
 *   gb_profile  runs the same work `iters` times as individual launches with
 *               CUDA events around each one, and accumulates per kernel class
 *               (GB_K_*) the device time ms[GB_NKCLASS] and launch count.
 */
int gb_replay(gb_handle *h, int iters, int with_grad, double *ms);
int gb_profile(gb_handle *h, int iters, int with_grad, double *ms, int *launches);

/*
 * Tuning knobs of the split-precision path (no counterpart in the reference),
 * set before the first evaluation of a handle or batch (GB_ERR_STATE after):
 *   GB_TUNE_MMA      0: mma.sync contractions, 1: tcgen05 (default)
 *   GB_TUNE_PERSIST  0: one launch per tree level, 1: persistent task-list
 *                    kernels (default; tcgen05 only)
 *   GB_TUNE_GCHUNK   patterns per partial sum of dlnL/dP (multiple of 64 in
 *                    [64, 8192]; default 2048, for a single alignment halved
 *                    down to 512 until there are four (pair, chunk) tasks per SM)
 *   GB_TUNE_ORDER    task order of the persistent kernels: 0 critical path
 *                    first (forward: deepest nodes below the root first;
 *                    adjoint: tallest subtrees first; all genes together;
 *                    default), 1 gene by gene by tree level, 2 by tree level
 *                    across genes
 *   GB_TUNE_GRID     CTAs per persistent launch (0: one per SM, the default)
 *   GB_TUNE_CHECKPOINT  FP64 handles, the adjoint's memory: 0 (default) keeps
 *                    every edge message E = P L~ of the forward and every
 *                    Ebar of the reverse sweep (3 + 3 blocks of the size of
 *                    the conditional likelihoods); 1 keeps the conditional
 *                    likelihoods of every internal node (the subtree roots
 *                    of the sweep) and recomputes the edge messages of one
 *                    tree level at a time during the reverse sweep, with the
 *                    dlnL/dP of that level's branches, so E and Ebar hold one
 *                    level (about half the device memory of a gradient
 *                    evaluation, one more forward pass of work; the same
 *                    arithmetic, so the same lnL and gradient bit for bit)
 * Environment defaults: GBCODEML_MMA=sync, GBCODEML_PERSIST=0.
 */
#define GB_TUNE_MMA     1
#define GB_TUNE_PERSIST 2
#define GB_TUNE_GCHUNK  3
#define GB_TUNE_ORDER   4
#define GB_TUNE_GRID    5
#define GB_TUNE_CHECKPOINT 6
int gb_tune(gb_handle *h, int knob, int value);
int gb_batch_tune(gb_batch *b, int knob, int value);

/*
 * Task trace of the persistent split-precision kernels (no counterpart in the
 * reference): with GBCODEML_TRACE=1 in the environment when the handle's
 * kernels are first set up, every task of the last evaluation records, from
 * the device's global timer, when it was claimed, when its dependencies were
 * met and when it ended, and the SM that ran it.  kernel: 0 pruning, 1 adjoint
 * propagation, 2 dlnL/dP.  Writes up to cap tasks, 12 words each (gene, item,
 * tile, edge (adjoint: the child edge a split item's task handles, -1 for the
 * whole item; 0 otherwise, as two's complement), claim ns, ready ns, four phase stamps (pruning: tips gathered,
 * first contraction's planes cut, its MMAs complete, its levels read; adjoint:
 * the same for its first contraction, the first stamp after the first child's
 * messages; 0 where a kernel records none), end ns, SM), and returns the
 * kernel's task count
 * (GB_ERR_STATE when tracing is off or the kernel has not run).
 */
int gb_task_trace(gb_handle *h, int kernel, unsigned long long *out, int cap);
/* the same for a batch's persistent kernels (gene = index in the batch) */
int gb_batch_task_trace(gb_batch *b, int kernel, unsigned long long *out, int cap);

/*
 * The persistent split-precision kernels' cross-CTA waits (a task waits for
 * the ready flags of the tiles it reads) are bounded: after wait_ms
 * milliseconds (0: the default, 2000) a waiting CTA sets the handle's error
 * word, stops claiming tasks, frees its tensor memory and returns, and the
 * evaluation returns GB_ERR_TIMEOUT.  withhold = 1 makes every such wait
 * expect a flag value that no task writes, so the next evaluations end that
 * way (a test of the error path that faults and hangs nothing); withhold = 0
 * restores normal evaluations on the same handle.  Needs a GB_PREC_FAST
 * handle whose persistent kernels have run (GB_ERR_STATE otherwise).  No
 * counterpart in the reference, which exits on any CUDA error
 * (cuda-codeml.cu:20-39).
 */
int gb_fault_inject(gb_handle *h, int wait_ms, int withhold);

/* Site models M7 (beta) and M8 (beta & omega_s): codeml's discretised
   beta, K equal-probability categories at their medians, omegas[j] =
   QuantileBeta((2j + 1) / (2K), p, q), props[j] = 1 / K (DiscreteNSsites
   codeml.c:2728-2770; M8 then scales props by p0 and adds omega_s with
   1 - p0).  Host only. */
int gb_beta_classes(double p, double q, int K, double *omegas, double *props);

/*
 * Host-only model set-up (no GPU needed): for codon frequencies pi[61] and
 * model-A parameters, the three eigen solutions U[i], V[i] (61x61 row-major),
 * Root[i] for w0, w1 = 1, w2, the Qfactors qf[2] and class proportions
 * freqK[4], as codeml's SetParametersNSsites computes them
 * (codeml.c:2488-2521, eigenQcodon codeml.c:3103-3273).  Each output may be
 * NULL.  U, V, Root point to arrays of 3*61*61, 3*61*61 and 3*61 doubles.
 */
int gb_model_setup(const double *pi, double kappa, double omega0, double omega2, double p0,
                   double p1, double *U, double *V, double *Root, double *qf, double *freqK);

/*
 * gb_lnL_noalloc -- no counterpart in the reference.  The FP64 lnL of
 * gb_eval_uvr for callers that cannot allocate device memory: their GPU
 * memory is owned by another allocator (an application pool or arena that
 * forbids outside allocations), or they cannot afford cudaMalloc/cudaFree,
 * which synchronise the whole device.  This call allocates nothing, on the
 * device or the host; its scratch is one static device array of
 * GB_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until
 * the process exits.  Problems needing more scratch (roughly npair * 32 KiB +
 * nslot * npad * 512 B, i.e. tens of taxa and a few thousand patterns at
 * most) are rejected with GB_ERR_ARG; at most 256 nodes.
 *   Host arrays: father[nnode], label[nnode], node_scale[nnode] (may be NULL:
 *   codeml's rule).  Device-accessible arrays owned by the caller: d_z
 *   [ns*npatt] codon ids, d_fpatt [npatt], d_pi [61], d_model
 *   [GB_MODEL_DOUBLES] = U[3][61*61], V[3][61*61], Root[3][61], qfactor[2],
 *   freqK[4] (the arrays gb_eval_uvr takes, concatenated), d_blength
 *   [nnode] (not checked: negative lengths act as 0); outputs d_neg_lnL [1]
 *   and d_fhK [4*npatt] (may be NULL).
 *   stream: a cudaStream_t (NULL = legacy default stream); the call returns
 *   after that stream has finished the evaluation.
 * Codon ids in d_z are checked on the device before any kernel uses them: an
 * id outside 0..60 gives GB_ERR_ARG and leaves the outputs untouched.
 * The first call on a device (with it current) looks up the scratch array's
 * device address and caches it for the process: do not use this entry point
 * across a cudaDeviceReset.  It cannot be called on a stream that is being
 * captured into a CUDA graph (GB_ERR_STATE): it synchronises the stream.  All
 * calls share the array: calls that overlap on the GPU race, so serialise them.
 */
#define GB_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
#define GB_MODEL_DOUBLES (6 * 61 * 61 + 3 * 61 + 2 + 4)
int gb_lnL_noalloc(int ns, int nnode, int root, const int *father, const int *label,
                   const char *node_scale, int npatt, const unsigned char *d_z,
                   const double *d_fpatt, const double *d_pi, const double *d_model,
                   const double *d_blength, double *d_neg_lnL, double *d_fhK, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GBCODEML_H */
