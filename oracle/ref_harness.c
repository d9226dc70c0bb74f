/*
 * ref_harness.c -- test infrastructure, not product code.
 *
 * Linked into the reference codeml builds of oracle/Makefile with
 * -Wl,--wrap=ming2: codeml.c's call of its optimiser (codeml.c:683-692, a
 * call into tools.c, another translation unit) lands in __wrap_ming2 with
 * codeml's own objective, its parameter vector x (in.codeml or codeml's
 * initial values, in codeml's own x space) and bounds, after codeml has read
 * the data, compressed the patterns and, in a CUDA build, run CUDA_Init.
 * Nothing in codeml.c, treesub.c or tools.c is changed.
 *
 * GBREF_MODE selects what happens there:
 *   (unset)  ming2 runs unchanged (the binary is codeml).
 *   time     GBREF_WARMUP + GBREF_STEPS steps, each one lnL and one gradient
 *            as ming2's first iteration forms it (tools.c:6396-6409): f0 =
 *            fun(x), then gradientB (tools.c:6326-6350) with SIZEp > 1, i.e.
 *            forward differences, np more evaluations of fun.  fun is
 *            codeml's lfundG (CPU build), the reference's CUDA_lfundG
 *            (CuCodeML build) or CUDA_lfundG over the drop-in adapter.
 *            GBREF_COORDS="first:count" restricts a step to f0 and the
 *            forward differences of those coordinates (gradientB's forward
 *            branch, tools.c:6342-6346), so that several processes can share
 *            one gradient.  Prints one line "GBREF {json}" with the per-step
 *            wall times, then exits.
 *   eval     prints fun(x) and codeml's CPU objective com.plfun(x) at the
 *            same x, codeml's central-difference gradient of com.plfun
 *            (gradientB with AlwaysCenter), a five-point stencil of
 *            com.plfun (step 1e-4 (|x_i| + 0.05)), and with GBREF_DFUN=1 where the
 *            adapter's GB_dfun is linked in (model A), its analytic gradient
 *            at x; then exits.
 *   dump     prints the data as codeml holds it after pattern compression
 *            and encoding (com.z with its ambiguity codes, com.fpatt, com.pi,
 *            nChara / CharaMap of SetMapAmbiguity treesub.c:1146-1200); then
 *            exits.
 *   sites    at x as final values (LASTROUND = 1), the adapter's GB_BEB and
 *            GB_HessianSKT2004 with codeml's SE arithmetic after it; prints
 *            the BEB arrays, log f(X) and the SEs, then exits.
 *   dfun     runs ming2 with the adapter's GB_dfun as its gradient hook
 *            (the one-argument change at codeml.c:688 that the drop-in
 *            enables), then codeml continues as usual.
 */
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#include <string.h>
#include <time.h>

#include "paml.h"
#include "codeml.h"

typedef double (*objective_t)(double x[], int n);
typedef int (*gradient_t)(double x[], double *f, double dx[], int n);

int __real_ming2(FILE *fout, double *f, objective_t fun, gradient_t dfun, double x[], double xb[][2],
                 double space[], double e, int n);
int gradientB(int n, double x[], double f0, double g[], objective_t fun, double space[], int xmark[]);

extern double SIZEp;
extern int AlwaysCenter;
extern int NFunCall;
extern double Small_Diff;

/* present only when the drop-in adapter is linked in */
extern int GB_dfun(double x[], double *f, double dx[], int n) __attribute__((weak));
extern int GB_BEB(double x[], int np, double postSite[], double grid[], double p0p1[], double lnfX[])
    __attribute__((weak));
extern int GB_HessianSKT2004(double xmle[], double lnLm, double g[], double H[]) __attribute__((weak));
extern int LASTROUND;
int matinv(double x[], int n, int m, double space[]);

static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

static int env_int(const char *name, int dflt) {
    const char *v = getenv(name);
    return v && *v ? atoi(v) : dflt;
}

static void print_vec(const char *key, const double *v, int n) {
    int i;
    printf("\"%s\": [", key);
    for (i = 0; i < n; i++) printf("%s%.17g", i ? ", " : "", v[i]);
    printf("]");
}

static void mode_time(objective_t fun, double x[], int n) {
    int i, s, warm = env_int("GBREF_WARMUP", 1), steps = env_int("GBREF_STEPS", 1), first = 0, count = -1;
    const char *co = getenv("GBREF_COORDS");
    double *g = (double *)calloc(n, sizeof(double)), *tv = (double *)malloc(sizeof(double) * 2 * n);
    double *t = (double *)malloc(sizeof(double) * (steps + 1)), f0 = 0;
    int *xmark = (int *)calloc(n, sizeof(int)), calls0 = NFunCall;
    if (!g || !tv || !t || !xmark) { fprintf(stderr, "ref_harness: out of memory\n"); exit(2); }
    if (co && *co && sscanf(co, "%d:%d", &first, &count) != 2) { fprintf(stderr, "ref_harness: GBREF_COORDS\n"); exit(2); }
    if (count >= 0 && (first < 0 || first + count > n)) { fprintf(stderr, "ref_harness: coordinates out of range\n"); exit(2); }
    for (s = -warm; s < steps; s++) {
        double t0 = now_s();
        calls0 = NFunCall;
        f0 = fun(x, n);
        SIZEp = 99;                     /* ming2's state before its first gradient */
        if (count < 0) {
            gradientB(n, x, f0, g, fun, tv, xmark);
        } else {
            for (i = first; i < first + count; i++) {   /* gradientB's forward branch */
                double eh = Small_Diff * (fabs(x[i]) + 1), *x1 = tv + n;
                memcpy(x1, x, sizeof(double) * n);
                x1[i] += eh;
                g[i] = (fun(x1, n) - f0) / eh;
            }
        }
        if (s >= 0) t[s] = now_s() - t0;
    }
    printf("\nGBREF {\"mode\": \"time\", \"np\": %d, \"npatt\": %d, \"ns\": %d, \"steps\": %d, \"warmup\": %d, "
           "\"coords\": [%d, %d], \"fun_calls_per_step\": %d, \"f0\": %.17g, ", n, com.npatt, com.ns, steps, warm,
           count < 0 ? 0 : first, count < 0 ? n : count, NFunCall - calls0, f0);
    print_vec("step_s", t, steps);
    printf(", ");
    print_vec("grad", g, n);
    printf("}\n");
    fflush(stdout);
    free(g); free(tv); free(t); free(xmark);
}

static void mode_eval(objective_t fun, double x[], int n) {
    double *g = (double *)malloc(sizeof(double) * n), *tv = (double *)malloc(sizeof(double) * 2 * n);
    double *ga = (double *)malloc(sizeof(double) * n), f_fun, f_cpu, fa = 0;
    double *g5 = (double *)calloc(n, sizeof(double));
    int i;
    int *xmark = (int *)calloc(n, sizeof(int)), have = GB_dfun != NULL && env_int("GBREF_DFUN", 0);
    if (!g || !tv || !ga || !g5 || !xmark) { fprintf(stderr, "ref_harness: out of memory\n"); exit(2); }
    f_fun = fun(x, n);
    f_cpu = com.plfun(x, n);
    if (have) GB_dfun(x, &fa, ga, n);
    AlwaysCenter = 1;
    gradientB(n, x, f_cpu, g, com.plfun, tv, xmark);
    /* a five-point stencil of the same CPU objective, step 1e-4 (|x_i| + 0.05):
       truncation O(h^4), an accurate derivative of codeml's own lnL */
    for (i = 0; i < n; i++) {
        static const int k[4] = {-2, -1, 1, 2};
        double f[4], h = 1e-4 * (fabs(x[i]) + 0.05), *x1 = tv + n;
        int q;
        for (q = 0; q < 4; q++) {
            memcpy(x1, x, sizeof(double) * n);
            x1[i] += k[q] * h;
            f[q] = com.plfun(x1, n);
        }
        g5[i] = (f[0] - 8 * f[1] + 8 * f[2] - f[3]) / (12 * h);
    }
    printf("\nGBREF {\"mode\": \"eval\", \"np\": %d, \"npatt\": %d, \"ns\": %d, \"f_fun\": %.17g, "
           "\"f_cpu\": %.17g, ", n, com.npatt, com.ns, f_fun, f_cpu);
    print_vec("x", x, n);
    printf(", ");
    print_vec("grad_cpu_central", g, n);
    printf(", ");
    print_vec("grad_cpu_5pt", g5, n);
    if (have) {
        printf(", \"f_dfun\": %.17g, ", fa);
        print_vec("grad_dfun", ga, n);
    }
    printf("}\n");
    fflush(stdout);
    free(g); free(tv); free(ga); free(g5); free(xmark);
}

/* what codeml computes after a model-A fit, through the adapter: at x taken
   as final values (LASTROUND = 1, so that SetParameters leaves Qfactor_NS_branch
   as codeml's BEB reads it), GB_BEB (the lfunNSsites_ACD arrays,
   codeml.c:6697-6775) and GB_HessianSKT2004 (codeml.c:764) followed by
   codeml's own SE arithmetic (H negated, matinv, sqrt of the diagonal,
   codeml.c:778-782) */
static void mode_sites(objective_t fun, double x[], int n) {
    /* clade models (model = 3): three classes, grid rows p0, p1, w0, [w1], w2, w3 */
    const int clade = com.model == 3, ncls = clade ? 3 : 4, ngrid = clade ? 10 * (5 + (com.NSsites == 3)) : 40;
    const int np4 = ncls * com.npatt;
    double *post = (double *)malloc(sizeof(double) * 4 * com.npatt), grid[60], p0p1[100], lnfX[3];
    double *g = (double *)malloc(sizeof(double) * n), *H = (double *)malloc(sizeof(double) * (2 * n * n + n));
    double f, se;
    int i;
    if (!GB_BEB || !GB_HessianSKT2004) { fprintf(stderr, "ref_harness: GBREF_MODE=sites needs the drop-in adapter\n"); exit(2); }
    if (!post || !g || !H) { fprintf(stderr, "ref_harness: out of memory\n"); exit(2); }
    LASTROUND = 1;
    f = fun(x, n);
    GB_BEB(x, n, post, grid, p0p1, lnfX);
    GB_HessianSKT2004(x, -f, g, H);
    for (i = 0; i < n * n; i++) H[i] *= -1;
    matinv(H, n, n, H + n * n);
    printf("\nGBREF {\"mode\": \"sites\", \"np\": %d, \"npatt\": %d, \"ncls\": %d, \"f\": %.17g, ", n,
           com.npatt, ncls, f);
    print_vec("post", post, np4);
    printf(", ");
    print_vec("grid", grid, ngrid);
    printf(", ");
    print_vec("p0p1", p0p1, 100);
    printf(", ");
    print_vec("lnfX", lnfX, 3);
    printf(", \"se\": [");
    for (i = 0; i < n; i++) {
        se = H[i * n + i] > 0. ? sqrt(H[i * n + i]) : -1;
        printf("%s%.17g", i ? ", " : "", se);
    }
    printf("]}\n");
    fflush(stdout);
    free(post); free(g); free(H);
}

static void mode_dump(void) {
    int j, h, c, k, maxcode = 0;
    printf("\nGBREF {\"mode\": \"dump\", \"ns\": %d, \"npatt\": %d, \"cleandata\": %d, \"z\": [",
           com.ns, com.npatt, (int)com.cleandata);
    for (j = 0; j < com.ns; j++) {
        printf("%s[", j ? ", " : "");
        for (h = 0; h < com.npatt; h++) {
            printf("%s%d", h ? ", " : "", (int)com.z[j][h]);
            if ((int)com.z[j][h] > maxcode) maxcode = com.z[j][h];
        }
        printf("]");
    }
    printf("], ");
    print_vec("fpatt", com.fpatt, com.npatt);
    printf(", ");
    print_vec("pi", com.pi, com.ncode);
    printf(", \"nchara\": [");
    for (c = 0; c <= maxcode; c++) printf("%s%d", c ? ", " : "", (int)nChara[c]);
    printf("], \"charamap\": [");
    for (c = 0; c <= maxcode; c++) {
        printf("%s[", c ? ", " : "");
        for (k = 0; k < nChara[c]; k++) printf("%s%d", k ? ", " : "", (int)CharaMap[c][k]);
        printf("]");
    }
    printf("]}\n");
    fflush(stdout);
}

int __wrap_ming2(FILE *fout, double *f, objective_t fun, gradient_t dfun, double x[], double xb[][2],
                 double space[], double e, int n) {
    const char *mode = getenv("GBREF_MODE");
    if (mode && !strcmp(mode, "time")) {
        mode_time(fun, x, n);
        exit(0);
    }
    if (mode && !strcmp(mode, "eval")) {
        mode_eval(fun, x, n);
        exit(0);
    }
    if (mode && !strcmp(mode, "dump")) {
        mode_dump();
        exit(0);
    }
    if (mode && !strcmp(mode, "sites")) {
        mode_sites(fun, x, n);
        exit(0);
    }
    /* a full fit: ming2 as codeml calls it (finite differences) or with
       GB_dfun; on stderr its wall time, iterations and lnL calls
       ("GBREF_MING2 seconds rounds calls") */
    if (mode && !strcmp(mode, "dfun")) {
        if (!GB_dfun) { fprintf(stderr, "ref_harness: GBREF_MODE=dfun needs the drop-in adapter\n"); exit(2); }
        dfun = GB_dfun;
    }
    {
        extern int Iround, NFunCall;
        const double t0 = now_s();
        const int calls0 = NFunCall;
        const int rc = __real_ming2(fout, f, fun, dfun, x, xb, space, e, n);
        fprintf(stderr, "GBREF_MING2 %.6f %d %d\n", now_s() - t0, Iround, NFunCall - calls0);
        return rc;
    }
}
