/*
 * codeml_adapter.c -- links into codeml in place of cuda-codeml.o.
 *
 * Compiled together with codeml's own sources (it needs codeml's paml.h and
 * codeml.h for the globals com, tree, nodes) and linked against
 * libgbcodeml.so; see include/gbcodeml_codeml.h for what each function
 * replaces.  It only marshals codeml's globals into the library's C ABI.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "paml.h"
#include "codeml.h"
#include "gbcodeml.h"
#include "gbcodeml_codeml.h"

/* codeml.c globals that are not declared in its headers */
extern double *_UU[NBTYPE + 2], *_VV[NBTYPE + 2], *_Root[NBTYPE + 2];
extern double Qfactor_NS_branch[NBTYPE];
extern int LASTROUND;
extern double Small_Diff;

static gb_handle *g_h = NULL;
static double *g_fhK = NULL;      /* [4*npatt] all classes of the current evaluation */
static double *g_blen = NULL;     /* [nnode] */
static int *g_bnode = NULL;       /* [nbranch] node of x[ib] */

static void gb_die(const char *what, int rc) {
    fprintf(stderr, "\ngbcodeml: %s failed (%d): %s\n", what, rc, gb_last_error());
    exit(-1);
}

/* a library handle (FP64) for codeml's current tree and data */
static gb_handle *make_handle(const char *who) {
    int i, j, rc;
    unsigned char *z;
    int *father, *label;
    char *scale = NULL;
    gb_problem p;
    gb_handle *h = NULL;
    /* codeml itself runs no branch-site or clade model on several genes
       (codeml.c:357); gaps and ambiguous codons (cleandata = 0) go to
       gb_create_unclean with codeml's own nChara / CharaMap */
    if (com.ngene != 1) gb_die(who, GB_ERR_ARG);
    if (com.ncode != GB_NCODE) gb_die(who, GB_ERR_ARG);
    z = (unsigned char *)malloc((size_t)com.ns * com.npatt);
    father = (int *)malloc(sizeof(int) * tree.nnode);
    label = (int *)malloc(sizeof(int) * tree.nnode);
    if (!z || !father || !label) gb_die(who, GB_ERR_OOM);
    for (j = 0; j < com.ns; j++) memcpy(z + (size_t)j * com.npatt, com.z[j], com.npatt);
    for (i = 0; i < tree.nnode; i++) {
        father[i] = nodes[i].father;
        label[i] = (i == tree.root) ? 0 : (int)nodes[i].label;
    }
    if (com.NnodeScale) scale = com.nodeScale;
    p.ns = com.ns;
    p.nnode = tree.nnode;
    p.root = tree.root;
    p.father = father;
    p.label = label;
    p.npatt = com.npatt;
    p.z = z;
    p.fpatt = com.fpatt;
    p.pi = com.pi;
    p.node_scale = scale;
    p.precision = GB_PREC_FP64;
    p.device = 0;
    if (!scale) {   /* codeml scales no node: tell the library so, rather than its own rule */
        scale = (char *)calloc(tree.nnode, 1);
        p.node_scale = scale;
    }
    rc = com.cleandata ? gb_create(&p, &h)
                       : gb_create_unclean(&p, (const unsigned char *)nChara, (const unsigned char *)CharaMap, &h);
    if (scale && scale != com.nodeScale) free(scale);
    free(z);
    free(father);
    free(label);
    if (rc) gb_die("gb_create", rc);
    return h;
}

void CUDA_Init(double *x) {
    int i;
    (void)x;
    /* the models whose site classes map onto the library's: branch-site A, B
       (model = 2) and clade C, D with two branch types (model = 3); codeml's
       other models never set up the per-class eigen slots this reads */
    if (!((com.model == 2 || (com.model == 3 && com.nbtype == 2)) && (com.NSsites == 2 || com.NSsites == 3)))
        gb_die("CUDA_Init (branch-site models A/B or clade models C/D with two branch types only)", GB_ERR_ARG);
    g_blen = (double *)malloc(sizeof(double) * tree.nnode);
    g_bnode = (int *)malloc(sizeof(int) * tree.nnode);
    g_fhK = (double *)malloc(sizeof(double) * 4 * com.npatt);
    if (!g_blen || !g_bnode || !g_fhK) gb_die("CUDA_Init (host memory)", GB_ERR_OOM);
    for (i = 0; i < tree.nnode; i++)
        if (i != tree.root) g_bnode[nodes[i].ibranch] = i;
    g_h = make_handle("CUDA_Init (one gene, universal code only)");
}

void CUDA_ScheduleConditionalPNode(int ir, int ig, double *x) {
    int i, rc;
    const int clade = com.model == 3;    /* clade models C / D (NSbranch3) */
    (void)x;
    if (ir == 0) {   /* SetParameters ran in CUDA_fx_r: U, V, Root, Qfactor, freqK are current */
        if (clade && (com.nbtype != 2 || com.ncatG != 3)) gb_die("clade model (two branch types only)", GB_ERR_ARG);
        for (i = 0; i < tree.nnode; i++)
            g_blen[i] = (i == tree.root) ? 0 : nodes[i].branch * com.rgene[ig];
        if (clade) {
            /* three classes, four eigen solutions: class 2 takes w2 on branch
               type 0 and w3 on type 1 (Set_UVR_BranchSite codeml.c:2561-2563) */
            rc = gb_eval_clade_uvr(g_h, (const double *const *)_UU, (const double *const *)_VV,
                                   (const double *const *)_Root, Qfactor_NS_branch, com.freqK, g_blen, NULL, g_fhK,
                                   NULL, NULL);
            if (rc) gb_die("gb_eval_clade_uvr", rc);
        } else {
            rc = gb_eval_uvr(g_h, (const double *const *)_UU, (const double *const *)_VV,
                             (const double *const *)_Root, Qfactor_NS_branch, com.freqK, g_blen, NULL, g_fhK,
                             NULL, NULL);
            if (rc) gb_die("gb_eval_uvr", rc);
        }
    }
    memcpy(com.fhK + (size_t)ir * com.npatt, g_fhK + (size_t)ir * com.npatt, sizeof(double) * com.npatt);
}

void CUDA_FreeAll(void) {
    if (g_h) gb_destroy(g_h);
    g_h = NULL;
    free(g_fhK);
    free(g_blen);
    free(g_bnode);
    g_fhK = g_blen = NULL;
    g_bnode = NULL;
}

int GB_dfun(double x[], double *f, double dx[], int n) {
    int rc;
    if (com.model == 3) {      /* clade models C (NSsites = 2) and D (NSsites = 3) */
        rc = gb_dfun_clade_x(g_h, g_bnode, LASTROUND, com.NSsites == 3, x, n, f, dx);
        if (rc) gb_die("gb_dfun_clade_x", rc);
        return 0;
    }
    rc = gb_dfun_x(g_h, g_bnode, LASTROUND, x, n, f, dx);
    if (rc) gb_die("gb_dfun_x", rc);
    return 0;
}

int GB_BEB(double x[], int np, double postSite[], double grid[], double p0p1[], double lnfX[]) {
    int i, rc;
    gb_handle *h;
    double *bl;
    if (np < com.ntime + 1) gb_die("GB_BEB (parameter vector)", GB_ERR_ARG);
    if (!(com.model == 2 || (com.model == 3 && com.nbtype == 2)))
        gb_die("GB_BEB (branch-site models A and B, clade models C and D with two branch types)", GB_ERR_ARG);
    bl = (double *)calloc(tree.nnode, sizeof(double));
    if (!bl) gb_die("GB_BEB (host memory)", GB_ERR_OOM);
    for (i = 0; i < tree.nnode; i++)
        if (i != tree.root) bl[i] = x[nodes[i].ibranch];
    h = make_handle("GB_BEB (one gene, universal code only)");
    /* kappa from x, the Qfactors of the last SetParameters (at the MLE), as
       codeml's BEB reads them (GetPMatBranch treesub.c:7289-7301) */
    if (com.model == 2) {
        /* models A and B: model A's grid; postSite[4*npatt], grid rows w0, w2 at [20..39] */
        rc = gb_beb_qf(h, bl, x[com.ntime], Qfactor_NS_branch, NULL, postSite, grid, p0p1, lnfX, NULL, NULL, NULL);
    } else {
        /* clade models C and D: postSite[3*npatt]; grid as lfunNSsites_ACD's
           postpara rows (dim x 10): p0, p1 (-1, ternary), w0, [w1 under D], w2, w3 */
        const int d = com.NSsites == 3, dim = 5 + d;
        double g4[40];
        int k, r;
        rc = gb_beb_clade_bl(h, d, bl, x[com.ntime], Qfactor_NS_branch, postSite, g4, p0p1, lnfX, NULL);
        for (r = 0; r < dim; r++)
            for (k = 0; k < 10; k++) {
                const int src = r < 2 ? -1 : (r == 2 ? 0 : (d && r == 3 ? 1 : r - 3 - d + 2));
                grid[r * 10 + k] = src < 0 ? -1.0 : g4[src * 10 + k];
            }
    }
    gb_destroy(h);
    free(bl);
    if (rc) gb_die("gb_beb", rc);
    return 0;
}

int GB_HessianSKT2004(double xmle[], double lnLm, double g[], double H[]) {
    int ib, rc;
    int *bnode;
    gb_handle *h;
    const int n = com.np;
    (void)lnLm;
    const int clade = com.model == 3;
    if (!((com.model == 2 && (n == com.ntime + 5 || n == com.ntime + 6)) ||
          (clade && com.nbtype == 2 && n == com.ntime + (com.NSsites == 3 ? 7 : 6))))
        gb_die("GB_HessianSKT2004 (branch-site models A and B, clade models C and D)", GB_ERR_ARG);
    bnode = (int *)malloc(sizeof(int) * tree.nnode);
    if (!bnode) gb_die("GB_HessianSKT2004 (host memory)", GB_ERR_OOM);
    for (ib = 0; ib < tree.nnode; ib++)
        if (ib != tree.root) bnode[nodes[ib].ibranch] = ib;
    h = make_handle("GB_HessianSKT2004 (one gene, universal code only)");
    rc = clade ? gb_se_opg_clade(h, bnode, com.NSsites == 3, xmle, n, Small_Diff, g, H, NULL)
               : gb_se_opg(h, bnode, xmle, n, Small_Diff, g, H, NULL, NULL);
    gb_destroy(h);
    free(bnode);
    if (rc) gb_die("gb_se_opg", rc);
    return 0;
}
