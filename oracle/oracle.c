/*
 * oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle; never shipped, never the
 * measured product path).  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load this library.
 *
 * A plain-C restatement of PAML codeml's branch-site model A likelihood path,
 * written from the algorithm in the reference sources, used as the FP64
 * checker for the CUDA library.  Each routine names the reference routine it
 * restates (paths relative to the reference project):
 *
 *   oracle_patterns   PatternWeight treesub.c:1302-1439 + EncodeSeqs
 *                     treesub.c:1075-1143 (clean codon data) + F3x4 codon
 *                     frequencies CountCodons/Fcodon_3x4 codeml.c:3475-3570,
 *                     InitializeCodon codeml.c:3732-3742
 *   build_q           eigenQcodon codeml.c:3103-3273 (GY94, HKY kappa, omega)
 *   eigen_uvr         eigenQREV tools.c:4850-4937 (symmetrisation with
 *                     sqrt(pi)); the symmetric eigenproblem is solved here by
 *                     cyclic Jacobi rotations instead of Householder+QL
 *                     (eigenRealSym tools.c:4943), an independent method
 *   set_params        SetParametersNSsites codeml.c:2381-2414, 2488-2521 and
 *                     f_and_x tools.c:1280-1305
 *   pmat              PMatUVRoot tools.c:515-546
 *   cond_node         ConditionalPNode codeml.c:3402-3459 (clean and unclean
 *                     tips: codeml's nChara / CharaMap, SetMapAmbiguity
 *                     treesub.c:1146-1200)
 *   node_scale        NodeScale treesub.c:6940-6975, SetNodeScale 6917-6937
 *   fx_r / lfundG     fx_r treesub.c:7485-7551, lfundG treesub.c:7342-7394
 *   gradientB         gradientB tools.c:6326-6350 (Small_Diff = 1e-6)
 *   oracle_beb        Bayes empirical Bayes site-class posteriors of model A:
 *                     lfunNSsites_ACD codeml.c:6617-6826,
 *                     get_grid_para_like_ACD 6419-6530, get_pclassM_iw_ACD
 *                     6532-6615, GetIndexTernary tools.c:4441-4461, and the
 *                     BEB branch of GetPMatBranch treesub.c:7289-7301
 *
 * The pattern loop is split over OpenMP threads (each thread walks the whole
 * tree for its own pattern range), which is the multi-core CPU baseline.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NC 61

static const char AA64[] =
    "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG";
static int g_sense[61];
static int g_init = 0;

static void init_code(void) {
    if (g_init) return;
    int n = 0;
    for (int i = 0; i < 64; i++)
        if (AA64[i] != '*') g_sense[n++] = i;
    g_init = 1;
}

/* ---------------------------------------------------------------- patterns */

static int g_ns, g_ncodon;
static const unsigned char *g_keys; /* [ncodon][3*ns] letter ranks */

static int cmp_site(const void *a, const void *b) {
    int ia = *(const int *)a, ib = *(const int *)b;
    int L = 3 * g_ns;
    int c = memcmp(g_keys + (size_t)ia * L, g_keys + (size_t)ib * L, L);
    if (c) return c;
    return ia < ib ? -1 : ia > ib;
}

/*
 * codons[ns*ncodon]: sense-codon index (0..60) per species and site.
 * Outputs: *npatt, z[ns*npatt] (codon id per species and pattern, row stride
 * npatt), fpatt[npatt], pi[61] (F3x4 from the data).  z and fpatt must hold
 * ncodon entries per species.  Patterns are ordered as codeml orders them:
 * by strcmp of the site's nucleotide letters (species-major, 3 per codon).
 */
int oracle_patterns(int ns, int ncodon, const int *codons, int *npatt_out,
                    unsigned char *z, double *fpatt, double *pi) {
    init_code();
    static const char BASES[] = "TCAG";
    /* rank of the letter under ASCII order: A < C < G < T */
    unsigned char rank[4];
    for (int b = 0; b < 4; b++) {
        unsigned char r = 0;
        for (int c = 0; c < 4; c++) r += (BASES[c] < BASES[b]);
        rank[b] = r;
    }
    int L = 3 * ns;
    unsigned char *keys = (unsigned char *)malloc((size_t)ncodon * L);
    int *idx = (int *)malloc(sizeof(int) * ncodon);
    if (!keys || !idx) return -1;
    for (int h = 0; h < ncodon; h++) {
        idx[h] = h;
        for (int j = 0; j < ns; j++) {
            int c = codons[(size_t)j * ncodon + h];
            if (c < 0 || c >= 61) { free(keys); free(idx); return -2; }
            int ic = g_sense[c];
            keys[(size_t)h * L + 3 * j + 0] = rank[ic / 16];
            keys[(size_t)h * L + 3 * j + 1] = rank[(ic / 4) % 4];
            keys[(size_t)h * L + 3 * j + 2] = rank[ic % 4];
        }
    }
    g_ns = ns; g_ncodon = ncodon; g_keys = keys;
    qsort(idx, ncodon, sizeof(int), cmp_site);
    int np = 0;
    for (int s = 0; s < ncodon; s++) {
        int h = idx[s];
        if (s == 0 || memcmp(keys + (size_t)h * L, keys + (size_t)idx[s - 1] * L, L) != 0) {
            for (int j = 0; j < ns; j++)
                z[(size_t)j * ncodon + np] = (unsigned char)codons[(size_t)j * ncodon + h];
            fpatt[np] = 0;
            np++;
        }
        fpatt[np - 1] += 1;
    }
    /* compact z rows to stride npatt */
    for (int j = 1; j < ns; j++)
        memmove(z + (size_t)j * np, z + (size_t)j * ncodon, np);
    *npatt_out = np;

    /* F3x4: codon counts (species then patterns, weighted by fpatt), then
       position x base table, then products over sense codons */
    double fcodon[64], fb[12];
    memset(fcodon, 0, sizeof fcodon);
    for (int j = 0; j < ns; j++)
        for (int h = 0; h < np; h++)
            fcodon[g_sense[z[(size_t)j * np + h]]] += fpatt[h];
    memset(fb, 0, sizeof fb);
    for (int k = 0; k < 64; k++) {
        int b0 = k / 16, b1 = (k % 16) / 4, b2 = k % 4;
        fb[0 * 4 + b0] += fcodon[k];
        fb[1 * 4 + b1] += fcodon[k];
        fb[2 * 4 + b2] += fcodon[k];
    }
    for (int j = 0; j < 3; j++) {
        double t = 0;
        for (int b = 0; b < 4; b++) t += fb[j * 4 + b];
        t = 1 / t;
        for (int b = 0; b < 4; b++) fb[j * 4 + b] *= t;
    }
    for (int i = 0; i < 61; i++) pi[i] = 0;
    for (int k = 0; k < 64; k++) {
        if (AA64[k] == '*') continue;
        int c = 0;
        while (g_sense[c] != k) c++;
        pi[c] = fb[k / 16] * fb[4 + (k / 4) % 4] * fb[8 + k % 4];
    }
    double s = 0;
    for (int i = 0; i < 61; i++) s += pi[i];
    s = 1 / s;
    for (int i = 0; i < 61; i++) pi[i] *= s;
    free(keys); free(idx);
    return 0;
}

/* --------------------------------------------------------------- Q, eigen */

/* GY94 Q (row i, column j), returns the mean rate -sum_i pi_i Q_ii. */
static double build_q(const double *pi, double kappa, double omega, double *Q) {
    init_code();
    for (int i = 0; i < NC * NC; i++) Q[i] = 0;
    for (int i = 1; i < NC; i++) {
        int ic1 = g_sense[i];
        int f[3] = {ic1 / 16, (ic1 / 4) % 4, ic1 % 4};
        for (int j = 0; j < i; j++) {
            int ic2 = g_sense[j];
            int t[3] = {ic2 / 16, (ic2 / 4) % 4, ic2 % 4};
            int ndiff = 0, pos = 0;
            for (int k = 0; k < 3; k++)
                if (f[k] != t[k]) { ndiff++; pos = k; }
            if (ndiff != 1) continue;
            double q = 1;
            if (f[pos] + t[pos] == 1 || f[pos] + t[pos] == 5) q = kappa;
            if (AA64[ic1] != AA64[ic2]) q *= omega;
            Q[i * NC + j] = q * pi[j];
            Q[j * NC + i] = q * pi[i];
        }
    }
    for (int i = 0; i < NC; i++) {
        double s = 0;
        for (int j = 0; j < NC; j++) s += Q[i * NC + j];
        Q[i * NC + i] = -s;
    }
    double mr = 0;
    for (int i = 0; i < NC; i++) mr -= pi[i] * Q[i * NC + i];
    return mr;
}

/* Cyclic Jacobi for a symmetric n x n matrix A (destroyed).  d: eigenvalues,
   R: eigenvectors in columns (R[i*n+k] is component i of vector k). */
static void jacobi(int n, double *A, double *d, double *R) {
    for (int i = 0; i < n * n; i++) R[i] = 0;
    for (int i = 0; i < n; i++) R[i * n + i] = 1;
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0, tot = 0;
        for (int p = 0; p < n; p++)
            for (int q = 0; q < n; q++) {
                double a = A[p * n + q] * A[p * n + q];
                tot += a;
                if (p != q) off += a;
            }
        if (off <= 1e-34 * tot || off == 0) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = A[p * n + q];
                if (fabs(apq) < 1e-300) continue;
                double app = A[p * n + p], aqq = A[q * n + q];
                double theta = (aqq - app) / (2 * apq);
                double t = (theta >= 0 ? 1 : -1) / (fabs(theta) + sqrt(theta * theta + 1));
                double c = 1 / sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    double rkp = R[k * n + p], rkq = R[k * n + q];
                    R[k * n + p] = c * rkp - s * rkq;
                    R[k * n + q] = s * rkp + c * rkq;
                }
            }
    }
    for (int i = 0; i < n; i++) d[i] = A[i * n + i];
}

/* Q = U diag(Root) V with V = U^-1; U = D^-1/2 R, V = R^T D^1/2. */
static void eigen_uvr(const double *Q, const double *pi, double *U, double *V, double *Root) {
    double A[NC * NC], R[NC * NC], sq[NC];
    for (int i = 0; i < NC; i++) sq[i] = sqrt(pi[i]);
    for (int i = 0; i < NC; i++) {
        A[i * NC + i] = Q[i * NC + i];
        for (int j = 0; j < i; j++)
            A[i * NC + j] = A[j * NC + i] = Q[i * NC + j] * sq[i] / sq[j];
    }
    jacobi(NC, A, Root, R);
    for (int i = 0; i < NC; i++)
        for (int k = 0; k < NC; k++) {
            U[i * NC + k] = R[i * NC + k] / sq[i];
            V[k * NC + i] = R[i * NC + k] * sq[i];
        }
}

/* ------------------------------------------------------------- the model */

typedef struct {
    int ns, nnode, root, npatt;
    const int *nson;          /* [nnode] */
    const int *sons;          /* [nnode*3] */
    const int *label;         /* [nnode] 0 background, 1 foreground */
    const int *bnode;         /* [nnode-1] node carrying x[ib] */
    const unsigned char *z;   /* [ns*npatt] */
    const double *fpatt;      /* [npatt] */
    const double *pi;         /* [61] */
    int nthreads;             /* <=0: all available */
    int model_b;              /* branch-site model B (NSsites = 3): w1 free, x = [..., w0, w1, w2] */
    const unsigned char *amb; /* NULL (clean data), or codeml's nChara[256] followed by
                                 CharaMap[256][64]: a tip code z >= 61 stands for the
                                 amb[z] sense codons amb[256 + 64 z + k] */
} oracle_problem;

typedef struct {
    double U[3][NC * NC], V[3][NC * NC], Root[3][NC];
    double qf[2], freqK[4];
    double kappa, w[3];
} params_t;

/* x = [t_0..t_{nb-1}, kappa, p0', p1', w0, w2] (model B: w0, w1, w2); p'
   are f_and_x-transformed unless lastround (then p0, p1 directly).  Model B
   (SetParametersNSsites codeml.c:2427-2436 with NSdiscrete) differs from A
   only in a free w1 where A fixes it at 1: in the site classes, the
   background / foreground mean rates behind the Qfactors and the second
   eigen solution. */
static int set_params(const oracle_problem *pb, const double *x, int lastround, params_t *P) {
    int nb = pb->nnode - 1, k = nb;
    double Q[NC * NC];
    P->kappa = x[k++];
    double f[3];
    if (!lastround) {
        double tot = 1;
        for (int i = 0; i < 2; i++) tot += (f[i] = exp(x[k + i]));
        for (int i = 0; i < 2; i++) f[i] /= tot;
        f[2] = 1 / tot;
        k += 2;
    } else {
        f[2] = 1;
        for (int i = 0; i < 2; i++) f[2] -= (f[i] = x[k++]);
    }
    P->freqK[0] = f[0]; P->freqK[1] = f[1]; P->freqK[2] = f[2];
    double w0 = x[k++], w1 = pb->model_b ? x[k++] : 1, w2 = x[k++];
    P->w[0] = w0; P->w[1] = w1; P->w[2] = w2;
    double t = P->freqK[0] + P->freqK[1];
    if (t < 1e-100) return -1;
    P->freqK[2] = (1 - t) * P->freqK[0] / t;
    P->freqK[3] = (1 - t) * P->freqK[1] / t;
    double wb[2][3] = {{w0, w1, -1}, {w0, w1, w2}};
    for (int i = 0; i < 2; i++) {
        double mr = 0;
        for (int j = 0; j < (i == 0 ? 2 : 3); j++) {
            double ff = P->freqK[j];
            if (i == 0) ff = P->freqK[j] / t;
            else if (j == 2) ff = 1 - t;
            mr += ff * wb[i][j];
        }
        P->qf[i] = 1 / build_q(pb->pi, P->kappa, mr, Q);
    }
    for (int i = 0; i < 3; i++) {
        build_q(pb->pi, P->kappa, P->w[i], Q);
        eigen_uvr(Q, pb->pi, P->U[i], P->V[i], P->Root[i]);
    }
    return 0;
}

/* P(t) row-major P[i*61+j] = sum_k U[i][k] e^{t Root_k} V[k][j], clamped >= 0 */
static void pmat(double *Pm, double t, const double *U, const double *V, const double *Root) {
    if (t < 1e-100) {
        for (int i = 0; i < NC * NC; i++) Pm[i] = 0;
        for (int i = 0; i < NC; i++) Pm[i * NC + i] = 1;
        return;
    }
    for (int i = 0; i < NC * NC; i++) Pm[i] = 0;
    for (int k = 0; k < NC; k++) {
        double e = exp(t * Root[k]);
        for (int i = 0; i < NC; i++) {
            double ue = U[i * NC + k] * e;
            double *row = Pm + i * NC;
            const double *vr = V + k * NC;
            for (int j = 0; j < NC; j++) row[j] += ue * vr[j];
        }
    }
    for (int i = 0; i < NC * NC; i++)
        if (Pm[i] < 0) Pm[i] = 0;
}

static int set_node_scale(const oracle_problem *pb, int inode, char *scale, int *nscale) {
    int d = 0;
    for (int i = 0; i < pb->nson[inode]; i++) {
        int s = pb->sons[inode * 3 + i];
        d += (pb->nson[s] ? set_node_scale(pb, s, scale, nscale) : 1);
    }
    if (inode != pb->root && d > 15) {
        scale[inode] = 1;
        d = 1;
        (*nscale)++;
    }
    return d;
}

typedef struct {
    const oracle_problem *pb;
    const double *Pall;     /* [nnode][61*61] for the current class */
    double *conP;           /* [nnode][npatt*61]; tips unused */
    const char *scale;
    double *scaleF;         /* [nnode][npatt] log scale (0 where unscaled) */
} walk_t;

static void cond_node(walk_t *w, int inode, int pos0, int pos1) {
    const oracle_problem *pb = w->pb;
    int n = NC, np = pb->npatt;
    for (int i = 0; i < pb->nson[inode]; i++) {
        int s = pb->sons[inode * 3 + i];
        if (pb->nson[s] > 0) cond_node(w, s, pos0, pos1);
    }
    double *cp = w->conP + (size_t)inode * np * n;
    for (int h = pos0 * n; h < pos1 * n; h++) cp[h] = 1;
    for (int i = 0; i < pb->nson[inode]; i++) {
        int s = pb->sons[inode * 3 + i];
        const double *Pm = w->Pall + (size_t)s * n * n;
        if (pb->nson[s] < 1) {
            const unsigned char *zs = pb->z + (size_t)s * np;
            for (int h = pos0; h < pos1; h++) {
                if (zs[h] < NC || !pb->amb) {
                    for (int j = 0; j < n; j++) cp[h * n + j] *= Pm[j * n + zs[h]];
                } else {
                    /* tip & unclean (ConditionalPNode codeml.c:3438-3445): the sum
                       over the sense codons the ambiguity code stands for */
                    const unsigned char *map = pb->amb + 256 + 64 * (size_t)zs[h];
                    for (int j = 0; j < n; j++) {
                        double t = 0;
                        for (int k = 0; k < pb->amb[zs[h]]; k++) t += Pm[j * n + map[k]];
                        cp[h * n + j] *= t;
                    }
                }
            }
        } else {
            const double *cs = w->conP + (size_t)s * np * n;
            for (int h = pos0; h < pos1; h++)
                for (int j = 0; j < n; j++) {
                    double t = 0;
                    for (int k = 0; k < n; k++) t += Pm[j * n + k] * cs[h * n + k];
                    cp[h * n + j] *= t;
                }
        }
    }
    if (w->scale[inode]) {
        double *sf = w->scaleF + (size_t)inode * np;
        for (int h = pos0; h < pos1; h++) {
            double t = 0;
            for (int j = 0; j < n; j++)
                if (cp[h * n + j] > t) t = cp[h * n + j];
            if (t < 1e-300) {
                for (int j = 0; j < n; j++) cp[h * n + j] = 1;
                sf[h] = -800;
            } else {
                for (int j = 0; j < n; j++) cp[h * n + j] /= t;
                sf[h] = log(t);
            }
        }
    }
}

/*
 * -lnL at x (codeml's lfundG value).  Optional outputs: fhK[4*npatt] as codeml
 * fills com.fhK (log f + sum of scale logs if any node is scaled, else f) and
 * lnf[npatt] = per-pattern log f (the values codeml writes to file lnf).
 * Returns NAN on a parameter error.
 */
double oracle_lnL(const oracle_problem *pb, const double *x, int lastround,
                  double *fhK_out, double *lnf_out, int *nscale_out) {
    int n = NC, np = pb->npatt, nn = pb->nnode;
    params_t *P = (params_t *)malloc(sizeof(params_t));
    if (set_params(pb, x, lastround, P)) { free(P); return NAN; }
    char *scale = (char *)calloc(nn, 1);
    int nscale = 0;
    set_node_scale(pb, pb->root, scale, &nscale);
    if (nscale_out) *nscale_out = nscale;
    double *Pall = (double *)malloc(sizeof(double) * nn * n * n);
    double *conP = (double *)malloc(sizeof(double) * (size_t)nn * np * n);
    double *scaleF = (double *)calloc((size_t)nn * np, sizeof(double));
    double *fhK = (double *)malloc(sizeof(double) * 4 * np);
    double *tnode = (double *)calloc(nn, sizeof(double));
    for (int ib = 0; ib < nn - 1; ib++) tnode[pb->bnode[ib]] = x[ib];
    int nth = pb->nthreads;
#ifdef _OPENMP
    if (nth <= 0) nth = omp_get_max_threads();
#else
    nth = 1;
#endif
    for (int ir = 0; ir < 4; ir++) {
        for (int i = 0; i < nn; i++) {
            if (i == pb->root) continue;
            int lab = pb->label[i];
            int iuvr = lab == 0 ? ir % 2 : (ir <= 1 ? ir : 2);
            pmat(Pall + (size_t)i * n * n, tnode[i] * P->qf[lab], P->U[iuvr], P->V[iuvr], P->Root[iuvr]);
        }
        walk_t w = {pb, Pall, conP, scale, scaleF};
        int chunks = nth * 4;
        if (chunks > np) chunks = np;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
        for (int c = 0; c < chunks; c++) {
            int pos0 = (int)((long)np * c / chunks), pos1 = (int)((long)np * (c + 1) / chunks);
            if (pos1 <= pos0) continue;
            cond_node(&w, pb->root, pos0, pos1);
            const double *cr = conP + (size_t)pb->root * np * n;
            for (int h = pos0; h < pos1; h++) {
                double fh = 0;
                for (int i = 0; i < n; i++) fh += pb->pi[i] * cr[h * n + i];
                if (fh <= 0) fh = 1e-300;
                if (!nscale) fhK[ir * np + h] = fh;
                else {
                    double v = log(fh);
                    for (int k = 0; k < nn; k++)
                        if (scale[k]) v += scaleF[(size_t)k * np + h];
                    fhK[ir * np + h] = v;
                }
            }
        }
    }
    double lnL = 0;
    for (int h = 0; h < np; h++) {
        double fh, t;
        if (pb->fpatt[h] <= 0) { if (lnf_out) lnf_out[h] = 0; continue; }
        if (nscale) {
            int it = 0;
            for (int ir = 1; ir < 4; ir++)
                if (fhK[ir * np + h] > fhK[it * np + h]) it = ir;
            t = fhK[it * np + h];
            fh = 0;
            for (int ir = 0; ir < 4; ir++) fh += P->freqK[ir] * exp(fhK[ir * np + h] - t);
            fh = t + log(fh);
        } else {
            fh = 0;
            for (int ir = 0; ir < 4; ir++) fh += P->freqK[ir] * fhK[ir * np + h];
            if (fh <= 0) fh = 1e-300;
            fh = log(fh);
        }
        lnL -= fh * pb->fpatt[h];
        if (lnf_out) lnf_out[h] = fh;
    }
    if (fhK_out) memcpy(fhK_out, fhK, sizeof(double) * 4 * np);
    free(P); free(scale); free(Pall); free(conP); free(scaleF); free(fhK); free(tnode);
    return lnL;
}

/* --------------------------------------------------------------- BEB */

#define BEB_D 10                                  /* grid points per dimension */
#define BEB_NW (BEB_D + 1 + BEB_D * BEB_D + BEB_D)  /* 121 omega sets */
#define BEB_NG (BEB_D * BEB_D * BEB_D * BEB_D)     /* (p0,p1) x w0 x w2 grid */

/* Root log f + scale logs for every pattern, one full pruning with the
   per-node transition matrices Pall (the root-sum step of fx_r,
   get_grid_para_like_ACD codeml.c:6504-6514: log taken whatever NnodeScale). */
static void root_logf(const oracle_problem *pb, const double *Pall, const char *scale, double *conP,
                      double *scaleF, double *out) {
    int n = NC, np = pb->npatt, nn = pb->nnode, nth = pb->nthreads;
#ifdef _OPENMP
    if (nth <= 0) nth = omp_get_max_threads();
#else
    nth = 1;
#endif
    walk_t w = {pb, Pall, conP, scale, scaleF};
    int chunks = nth * 4;
    if (chunks > np) chunks = np;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
    for (int c = 0; c < chunks; c++) {
        int pos0 = (int)((long)np * c / chunks), pos1 = (int)((long)np * (c + 1) / chunks);
        if (pos1 <= pos0) continue;
        cond_node(&w, pb->root, pos0, pos1);
        const double *cr = conP + (size_t)pb->root * np * n;
        for (int h = pos0; h < pos1; h++) {
            double fh = 0;
            for (int i = 0; i < n; i++) fh += pb->pi[i] * cr[h * n + i];
            if (fh <= 0) fh = 1e-300;
            fh = log(fh);
            for (int k = 0; k < nn; k++)
                if (scale[k]) fh += scaleF[(size_t)k * np + h];
            out[h] = fh;
        }
    }
}

/* omega index (0..9 grid w0, 10 = w1 = 1, 11..20 grid w2) of the background
   and foreground branches for omega set iw: 10 sets (w0, w0), 1 set (1, 1),
   100 sets (w0_i, w2_j) with iw = 11 + 10 i + j, 10 sets (1, w2_j). */
static void beb_omega_set(int iw, int *eb, int *ef) {
    if (iw < BEB_D) { *eb = *ef = iw; }
    else if (iw == BEB_D) { *eb = *ef = BEB_D; }
    else if (iw < BEB_D + 1 + BEB_D * BEB_D) {
        *eb = (iw - BEB_D - 1) / BEB_D;
        *ef = BEB_D + 1 + (iw - BEB_D - 1) % BEB_D;
    } else { *eb = BEB_D; *ef = BEB_D + 1 + (iw - BEB_D - 1 - BEB_D * BEB_D); }
}

/*
 * Bayes empirical Bayes under branch-site model A at x (normally the MLE).
 * The synonymous branch lengths stay at the MLE: Qfactor_NS_branch and kappa
 * come from x, while omega runs over the grid (w0 in (0,1), w2 in (1,11),
 * 10 points each) and (p0, p1) over 100 triangles of the ternary plot.
 * Outputs (each may be NULL):
 *   lnfw[121*npatt]  log f(x_h | omega set) before rescaling
 *   post[4*npatt]    posterior of the site classes 0, 1, 2a, 2b per pattern
 *   grid[4*10]       posterior of the grid values of p0, p1 (-1: not
 *                    computed), w0, w2 (codeml's "Posterior on the grid")
 *   p0p1[100]        posterior over the ternary (p0, p1) triangles
 *   lnfX[3]          log f(X) as codeml prints it, and its scale terms S1, S2
 *   wmean, wsd[npatt] posterior mean and SD of the site's w with classes 0,
 *                    1, 2a, 2b at w0_i, 1, w2_j, w2_j (M2a's "post mean +- SE
 *                    for w" on an all-foreground tree, lfunNSsites_M2M8
 *                    codeml.c:6331-6374)
 * Returns 0, or -1 on a parameter error.
 */
int oracle_beb(const oracle_problem *pb, const double *x, int lastround, double *lnfw_out,
               double *post, double *grid, double *p0p1, double *lnfX, double *wmean, double *wsd) {
    int n = NC, np = pb->npatt, nn = pb->nnode;
    params_t *P = (params_t *)malloc(sizeof(params_t));
    if (set_params(pb, x, lastround, P)) { free(P); return -1; }
    /* the 21 omega values and their eigen solutions (unscaled Q: eigenQcodon
       with meanrate 1, the Qfactor of the MLE applied to t) */
    double wv[2 * BEB_D + 1];
    for (int i = 0; i < BEB_D; i++) {
        wv[i] = (i + 0.5) / BEB_D;
        wv[BEB_D + 1 + i] = 1 + (i + 0.5) * (11 - 1) / BEB_D;
    }
    wv[BEB_D] = 1;
    int ne = 2 * BEB_D + 1;
    double *U = (double *)malloc(sizeof(double) * ne * n * n);
    double *V = (double *)malloc(sizeof(double) * ne * n * n);
    double *R = (double *)malloc(sizeof(double) * ne * n);
    double *Q = (double *)malloc(sizeof(double) * n * n);
    for (int e = 0; e < ne; e++) {
        build_q(pb->pi, P->kappa, wv[e], Q);
        eigen_uvr(Q, pb->pi, U + (size_t)e * n * n, V + (size_t)e * n * n, R + (size_t)e * n);
    }
    char *scale = (char *)calloc(nn, 1);
    int nscale = 0;
    set_node_scale(pb, pb->root, scale, &nscale);
    double *tnode = (double *)calloc(nn, sizeof(double));
    for (int ib = 0; ib < nn - 1; ib++) tnode[pb->bnode[ib]] = x[ib];
    double *Pall = (double *)malloc(sizeof(double) * nn * n * n);
    double *conP = (double *)malloc(sizeof(double) * (size_t)nn * np * n);
    double *scaleF = (double *)calloc((size_t)nn * np, sizeof(double));
    double *F = (double *)malloc(sizeof(double) * (size_t)BEB_NW * np);
    for (int iw = 0; iw < BEB_NW; iw++) {
        int eb, ef;
        beb_omega_set(iw, &eb, &ef);
        for (int i = 0; i < nn; i++) {
            if (i == pb->root) continue;
            int lab = pb->label[i], e = lab ? ef : eb;
            pmat(Pall + (size_t)i * n * n, tnode[i] * P->qf[lab], U + (size_t)e * n * n,
                 V + (size_t)e * n * n, R + (size_t)e * n);
        }
        root_logf(pb, Pall, scale, conP, scaleF, F + (size_t)iw * np);
    }
    if (lnfw_out) memcpy(lnfw_out, F, sizeof(double) * BEB_NW * np);
    /* per-pattern rescaling by the largest of the 121 values (S1) */
    double S1 = 0;
    for (int h = 0; h < np; h++) {
        double m = F[h];
        for (int k = 1; k < BEB_NW; k++)
            if (F[(size_t)k * np + h] > m) m = F[(size_t)k * np + h];
        for (int k = 0; k < BEB_NW; k++) F[(size_t)k * np + h] = exp(F[(size_t)k * np + h] - m);
        S1 += m * pb->fpatt[h];
    }
    /* grid: class proportions (ternary centroids, 2a/2b split p2 by p0:p1) and
       the omega set each class reads */
    double *pcl = (double *)malloc(sizeof(double) * BEB_NG * 4);
    int *iwg = (int *)malloc(sizeof(int) * BEB_NG * 4);
    for (int g = 0; g < BEB_NG; g++) {
        int ip[4];
        for (int j = 3, it = g; j >= 0; j--) { ip[j] = it % BEB_D; it /= BEB_D; }
        int t = ip[0] * BEB_D + ip[1];
        int ix = (int)sqrt((double)t), iy = t - ix * ix;
        double p[3];
        p[0] = (1 + (iy / 2) * 3 + (iy % 2)) / (3. * BEB_D);
        p[1] = (1 + (BEB_D - 1 - ix) * 3 + (iy % 2)) / (3. * BEB_D);
        p[2] = 1 - p[0] - p[1];
        pcl[g * 4 + 0] = p[0];
        pcl[g * 4 + 1] = p[1];
        pcl[g * 4 + 2] = p[2] * p[0] / (1 - p[2]);
        pcl[g * 4 + 3] = p[2] * p[1] / (1 - p[2]);
        iwg[g * 4 + 0] = ip[2];
        iwg[g * 4 + 1] = BEB_D;
        iwg[g * 4 + 2] = BEB_D + 1 + ip[2] * BEB_D + ip[3];
        iwg[g * 4 + 3] = BEB_D + 1 + BEB_D * BEB_D + ip[3];
    }
    /* marginal likelihood f(X) over the grid, with codeml's running scale S2 */
    double *lnfXs = (double *)malloc(sizeof(double) * BEB_NG);
    double pp[4][BEB_D], pq[BEB_D * BEB_D];
    memset(pp, 0, sizeof pp);
    memset(pq, 0, sizeof pq);
    double fX = 1, S2 = -1e300;
    for (int g = 0; g < BEB_NG; g++) {
        int ip[4];
        for (int j = 3, it = g; j >= 0; j--) { ip[j] = it % BEB_D; it /= BEB_D; }
        double s = 0;
        for (int h = 0; h < np; h++) {
            double fh = 0;
            for (int k = 0; k < 4; k++) fh += pcl[g * 4 + k] * F[(size_t)iwg[g * 4 + k] * np + h];
            if (fh < 1e-300) continue;
            s += log(fh) * pb->fpatt[h];
        }
        lnfXs[g] = s;
        double t = s - S2;
        if (t > 10) {
            t = t < 200 ? exp(-t) : 0;
            fX = fX * t + 1;
            for (int j = 0; j < 4; j++)
                for (int k = 0; k < BEB_D; k++) pp[j][k] *= t;
            for (int k = 0; k < BEB_D * BEB_D; k++) pq[k] *= t;
            for (int j = 0; j < 4; j++) pp[j][ip[j]] += 1;
            pq[ip[0] * BEB_D + ip[1]] += 1;
            S2 = s;
        } else if (t > -200) {
            t = exp(t);
            fX += t;
            for (int j = 0; j < 4; j++) pp[j][ip[j]] += t;
            pq[ip[0] * BEB_D + ip[1]] += t;
        }
    }
    for (int j = 0; j < 4; j++)
        for (int k = 0; k < BEB_D; k++) pp[j][k] /= fX;
    for (int k = 0; k < BEB_D * BEB_D; k++) pq[k] /= fX;
    double lfX = log(fX) + S2;
    if (lnfX) {
        lnfX[0] = lfX + S1 - 4 * log((double)BEB_D);
        lnfX[1] = S1;
        lnfX[2] = S2;
    }
    if (grid) {
        for (int k = 0; k < BEB_D; k++) grid[k] = grid[BEB_D + k] = -1;
        for (int j = 2; j < 4; j++)
            for (int k = 0; k < BEB_D; k++) grid[j * BEB_D + k] = pp[j][k];
    }
    if (p0p1) memcpy(p0p1, pq, sizeof pq);
    /* posterior of the four site classes per pattern */
    if (post) {
#pragma omp parallel for schedule(dynamic, 4)
        for (int h = 0; h < np; h++) {
            double acc[4] = {0, 0, 0, 0};
            for (int g = 0; g < BEB_NG; g++) {
                double fk[4], fh = 0;
                for (int k = 0; k < 4; k++)
                    fh += fk[k] = pcl[g * 4 + k] * F[(size_t)iwg[g * 4 + k] * np + h];
                for (int k = 0; k < 4; k++) {
                    double t = log(fk[k] / fh) + lnfXs[g] - lfX;
                    if (t > -300) acc[k] += exp(t);
                }
            }
            for (int k = 0; k < 4; k++) post[k * np + h] = acc[k];
        }
    }
    /* posterior mean and SD of w: terms exp(log(ratio w) + lnfXs - log f(X)),
       skipped where ratio w < 1e-300 (codeml.c:6358-6374) */
    if (wmean || wsd) {
#pragma omp parallel for schedule(dynamic, 4)
        for (int h = 0; h < np; h++) {
            double m1 = 0, m2 = 0;
            for (int g = 0; g < BEB_NG; g++) {
                int ip2 = (g / BEB_D) % BEB_D, ip3 = g % BEB_D;
                double om[4] = {wv[ip2], 1, wv[BEB_D + 1 + ip3], wv[BEB_D + 1 + ip3]};
                double fk[4], fh = 0;
                for (int k = 0; k < 4; k++)
                    fh += fk[k] = pcl[g * 4 + k] * F[(size_t)iwg[g * 4 + k] * np + h];
                for (int k = 0; k < 4; k++) {
                    double r = fk[k] / fh, a = r * om[k];
                    if (!(a >= 1e-300)) continue;
                    m1 += exp(log(a) + lnfXs[g] - lfX);
                    m2 += exp(log(a * om[k]) + lnfXs[g] - lfX);
                }
            }
            double v = m2 - m1 * m1;
            if (wmean) wmean[h] = m1;
            if (wsd) wsd[h] = v > 0 ? sqrt(v) : 0;
        }
    }
    free(P); free(U); free(V); free(R); free(Q); free(scale); free(tnode); free(Pall);
    free(conP); free(scaleF); free(F); free(pcl); free(iwg); free(lnfXs);
    return 0;
}

/*
 * Bayes empirical Bayes under clade model C with two branch types
 * (lfunNSsites_ACD codeml.c:6617-6826 with modelACD = mC; grid set-up
 * get_grid_para_like_ACD 6419-6470, classes get_pclassM_iw_ACD 6532-6615):
 * x = [branch lengths, kappa, p0, p1, w0, w2 (background), w3 (foreground)].
 * 111 omega sets: 10 (w0_i everywhere, w0 in (0, 1)), 1 (w = 1), and 100
 * (w2_i on background, w3_j on foreground, both in (0, 3)) with set index
 * 11 + 10 i + j; Qfactor_NS_branch of the two branch types fixed at x.  Grid:
 * 100 ternary (p0, p1) triangles x w0 x w2 x w3 (10^5 points), classes
 * (p0, p1, p2).  Outputs as oracle_beb: lnfw[111*npatt], post[3*npatt],
 * grid[5*10] (rows p0, p1 = -1, w0, w2, w3), p0p1[100], lnfX[3].
 */
int oracle_beb_clade(const oracle_problem *pb, const double *x, double *lnfw_out, double *post,
                     double *grid, double *p0p1, double *lnfX) {
    const int D = BEB_D, NW = D + 1 + D * D, DIM = 5;
    const long NG = (long)D * D * D * D * D;
    int n = NC, np = pb->npatt, nn = pb->nnode, nb = nn - 1;
    double kappa = x[nb], p0 = x[nb + 1], p1 = x[nb + 2], w0 = x[nb + 3], w2 = x[nb + 4], w3 = x[nb + 5];
    double p2 = 1 - p0 - p1, Q[NC * NC];
    double qf[2] = {1 / build_q(pb->pi, kappa, p0 * w0 + p1 + p2 * w2, Q),
                    1 / build_q(pb->pi, kappa, p0 * w0 + p1 + p2 * w3, Q)};
    /* omega values: 0..9 w0 grid, 10 = 1, 11..20 the (0, 3) grid of w2 and w3 */
    double wv[2 * BEB_D + 1];
    for (int i = 0; i < D; i++) {
        wv[i] = (i + 0.5) / D;
        wv[D + 1 + i] = 0 + (i + 0.5) * (3 - 0) / D;
    }
    wv[D] = 1;
    int ne = 2 * D + 1;
    double *U = (double *)malloc(sizeof(double) * ne * n * n), *V = (double *)malloc(sizeof(double) * ne * n * n);
    double *R = (double *)malloc(sizeof(double) * ne * n);
    for (int e = 0; e < ne; e++) {
        build_q(pb->pi, kappa, wv[e], Q);
        eigen_uvr(Q, pb->pi, U + (size_t)e * n * n, V + (size_t)e * n * n, R + (size_t)e * n);
    }
    char *scale = (char *)calloc(nn, 1);
    int nscale = 0;
    set_node_scale(pb, pb->root, scale, &nscale);
    double *tnode = (double *)calloc(nn, sizeof(double));
    for (int ib = 0; ib < nb; ib++) tnode[pb->bnode[ib]] = x[ib];
    double *Pall = (double *)malloc(sizeof(double) * nn * n * n);
    double *conP = (double *)malloc(sizeof(double) * (size_t)nn * np * n);
    double *scaleF = (double *)calloc((size_t)nn * np, sizeof(double));
    double *F = (double *)malloc(sizeof(double) * (size_t)NW * np);
    for (int iw = 0; iw < NW; iw++) {
        int eb, ef;
        if (iw < D) eb = ef = iw;
        else if (iw == D) eb = ef = D;
        else { eb = D + 1 + (iw - D - 1) / D; ef = D + 1 + (iw - D - 1) % D; }
        for (int i = 0; i < nn; i++) {
            if (i == pb->root) continue;
            int lab = pb->label[i], e = lab ? ef : eb;
            pmat(Pall + (size_t)i * n * n, tnode[i] * qf[lab], U + (size_t)e * n * n, V + (size_t)e * n * n,
                 R + (size_t)e * n);
        }
        root_logf(pb, Pall, scale, conP, scaleF, F + (size_t)iw * np);
    }
    if (lnfw_out) memcpy(lnfw_out, F, sizeof(double) * NW * np);
    double S1 = 0;
    for (int h = 0; h < np; h++) {
        double m = F[h];
        for (int k = 1; k < NW; k++)
            if (F[(size_t)k * np + h] > m) m = F[(size_t)k * np + h];
        for (int k = 0; k < NW; k++) F[(size_t)k * np + h] = exp(F[(size_t)k * np + h] - m);
        S1 += m * pb->fpatt[h];
    }
    double tri[100][3];
    for (int t = 0; t < 100; t++) {
        int ix = (int)sqrt((double)t), iy = t - ix * ix;
        tri[t][0] = (1 + (iy / 2) * 3 + (iy % 2)) / (3. * D);
        tri[t][1] = (1 + (D - 1 - ix) * 3 + (iy % 2)) / (3. * D);
        tri[t][2] = 1 - tri[t][0] - tri[t][1];
    }
    double *lnfXs = (double *)malloc(sizeof(double) * NG);
#pragma omp parallel for schedule(static)
    for (long g = 0; g < NG; g++) {
        int ip[5];
        long it = g;
        for (int j = 4; j >= 0; j--) { ip[j] = (int)(it % D); it /= D; }
        const double *pc = tri[ip[0] * D + ip[1]];
        const double *f0 = F + (size_t)ip[2] * np, *f1 = F + (size_t)D * np;
        const double *f2 = F + (size_t)(D + 1 + ip[3] * D + ip[4]) * np;
        double sum = 0;
        for (int h = 0; h < np; h++) {
            double fh = pc[0] * f0[h] + pc[1] * f1[h] + pc[2] * f2[h];
            if (fh < 1e-300) continue;
            sum += log(fh) * pb->fpatt[h];
        }
        lnfXs[g] = sum;
    }
    double pp[5][BEB_D], pq[100];
    memset(pp, 0, sizeof pp);
    memset(pq, 0, sizeof pq);
    double fX = 1, S2 = -1e300;
    for (long g = 0; g < NG; g++) {
        int ip[5];
        long it = g;
        for (int j = 4; j >= 0; j--) { ip[j] = (int)(it % D); it /= D; }
        double t = lnfXs[g] - S2;
        if (t > 10) {
            t = t < 200 ? exp(-t) : 0;
            fX = fX * t + 1;
            for (int j = 0; j < DIM; j++)
                for (int k = 0; k < D; k++) pp[j][k] *= t;
            for (int k = 0; k < 100; k++) pq[k] *= t;
            for (int j = 0; j < DIM; j++) pp[j][ip[j]] += 1;
            pq[ip[0] * D + ip[1]] += 1;
            S2 = lnfXs[g];
        } else if (t > -200) {
            t = exp(t);
            fX += t;
            for (int j = 0; j < DIM; j++) pp[j][ip[j]] += t;
            pq[ip[0] * D + ip[1]] += t;
        }
    }
    double lfX = log(fX) + S2;
    if (lnfX) {
        lnfX[0] = lfX + S1 - DIM * log((double)D);
        lnfX[1] = S1;
        lnfX[2] = S2;
    }
    if (grid)
        for (int j = 0; j < DIM; j++)
            for (int k = 0; k < D; k++) grid[j * D + k] = j < 2 ? -1 : pp[j][k] / fX;
    if (p0p1)
        for (int k = 0; k < 100; k++) p0p1[k] = pq[k] / fX;
    if (post) {
#pragma omp parallel for schedule(dynamic, 4)
        for (int h = 0; h < np; h++) {
            double acc[3] = {0, 0, 0};
            for (long g = 0; g < NG; g++) {
                int ip[5];
                long it = g;
                for (int j = 4; j >= 0; j--) { ip[j] = (int)(it % D); it /= D; }
                const double *pc = tri[ip[0] * D + ip[1]];
                double fk[3] = {pc[0] * F[(size_t)ip[2] * np + h], pc[1] * F[(size_t)D * np + h],
                                pc[2] * F[(size_t)(D + 1 + ip[3] * D + ip[4]) * np + h]};
                double fh = fk[0] + fk[1] + fk[2];
                for (int k = 0; k < 3; k++) {
                    double t = log(fk[k] / fh) + lnfXs[g] - lfX;
                    if (t > -300) acc[k] += exp(t);
                }
            }
            for (int k = 0; k < 3; k++) post[k * np + h] = acc[k];
        }
    }
    free(U); free(V); free(R); free(scale); free(tnode); free(Pall); free(conP); free(scaleF); free(F);
    free(lnfXs);
    return 0;
}

/*
 * Per-class fhK (as oracle_lnL writes it) from given eigen solutions: U, V
 * [3][61*61], Root [3][61] (model A's slots w0, w1, w2), Qfactors qf[2] and
 * branch lengths by branch index (x[0..nb-1]); the classes follow model A's
 * map (Set_UVR_BranchSite codeml.c:2555-2558).  Used to restate models whose
 * classes are model-A classes of different eigen slots (clade model C: its
 * third class is class 2a with slots (w2, -, w3)).  Returns nscale.
 */
int oracle_fhK_uvr(const oracle_problem *pb, const double *U, const double *V, const double *Root,
                   const double *qf, const double *xb, double *fhK) {
    int n = NC, np = pb->npatt, nn = pb->nnode;
    params_t *P = (params_t *)malloc(sizeof(params_t));
    for (int i = 0; i < 3; i++) {
        memcpy(P->U[i], U + i * NC * NC, sizeof(double) * NC * NC);
        memcpy(P->V[i], V + i * NC * NC, sizeof(double) * NC * NC);
        memcpy(P->Root[i], Root + i * NC, sizeof(double) * NC);
    }
    P->qf[0] = qf[0];
    P->qf[1] = qf[1];
    char *scale = (char *)calloc(nn, 1);
    int nscale = 0;
    set_node_scale(pb, pb->root, scale, &nscale);
    double *Pall = (double *)malloc(sizeof(double) * nn * n * n);
    double *conP = (double *)malloc(sizeof(double) * (size_t)nn * np * n);
    double *scaleF = (double *)calloc((size_t)nn * np, sizeof(double));
    double *tnode = (double *)calloc(nn, sizeof(double));
    double *lf = (double *)malloc(sizeof(double) * np);
    for (int ib = 0; ib < nn - 1; ib++) tnode[pb->bnode[ib]] = xb[ib];
    for (int ir = 0; ir < 4; ir++) {
        for (int i = 0; i < nn; i++) {
            if (i == pb->root) continue;
            int lab = pb->label[i];
            int iuvr = lab == 0 ? ir % 2 : (ir <= 1 ? ir : 2);
            pmat(Pall + (size_t)i * n * n, tnode[i] * P->qf[lab], P->U[iuvr], P->V[iuvr], P->Root[iuvr]);
        }
        root_logf(pb, Pall, scale, conP, scaleF, lf);
        for (int h = 0; h < np; h++) fhK[ir * np + h] = nscale ? lf[h] : exp(lf[h]);
    }
    free(P); free(scale); free(Pall); free(conP); free(scaleF); free(tnode); free(lf);
    return nscale;
}

/* Model quantities codeml derives from x, for parity tests of the CUDA
   library's own host set-up: U,V,Root (3 sets, 61x61 row-major), qf[2],
   freqK[4]. */
int oracle_set_params(const oracle_problem *pb, const double *x, int lastround,
                      double *U, double *V, double *Root, double *qf, double *freqK) {
    params_t *P = (params_t *)malloc(sizeof(params_t));
    int rc = set_params(pb, x, lastround, P);
    if (!rc) {
        for (int i = 0; i < 3; i++) {
            memcpy(U + i * NC * NC, P->U[i], sizeof(double) * NC * NC);
            memcpy(V + i * NC * NC, P->V[i], sizeof(double) * NC * NC);
            memcpy(Root + i * NC, P->Root[i], sizeof(double) * NC);
        }
        memcpy(qf, P->qf, sizeof(double) * 2);
        memcpy(freqK, P->freqK, sizeof(double) * 4);
    }
    free(P);
    return rc;
}

/* GY94 Q and its mean rate (eigenQcodon mode 0). */
double oracle_build_q(const double *pi, double kappa, double omega, double *Q) {
    return build_q(pi, kappa, omega, Q);
}

/* P(t) as PMatUVRoot computes it. */
void oracle_pmat(double *Pm, double t, const double *U, const double *V, const double *Root) {
    pmat(Pm, t, U, V, Root);
}

/*
 * codeml's numerical gradient of -lnL (gradientB with every xmark = 0 and
 * SIZEp < 1, i.e. central differences with step (1e-6 (|x_i|+1))^0.67).
 * central=0 gives the forward-difference form with step 1e-6 (|x_i|+1).
 */
int oracle_gradientB(const oracle_problem *pb, const double *x, int np_, int lastround,
                     int central, double *g) {
    double *x0 = (double *)malloc(sizeof(double) * np_);
    double *x1 = (double *)malloc(sizeof(double) * np_);
    double f0 = central ? 0 : oracle_lnL(pb, x, lastround, NULL, NULL, NULL);
    for (int i = 0; i < np_; i++) {
        double eh = 1e-6 * (fabs(x[i]) + 1);
        memcpy(x0, x, sizeof(double) * np_);
        memcpy(x1, x, sizeof(double) * np_);
        if (central) {
            eh = pow(eh, .67);
            x0[i] -= eh; x1[i] += eh;
            g[i] = (oracle_lnL(pb, x1, lastround, NULL, NULL, NULL) -
                    oracle_lnL(pb, x0, lastround, NULL, NULL, NULL)) / (eh * 2.0);
        } else {
            x1[i] += eh;
            g[i] = (oracle_lnL(pb, x1, lastround, NULL, NULL, NULL) - f0) / eh;
        }
    }
    free(x0); free(x1);
    return 0;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
