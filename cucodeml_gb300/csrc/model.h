// Host-side model A set-up: GY94 rate matrices, their eigen solutions, the
// branch-type Qfactors and site-class proportions, plus the derivative terms
// the adjoint needs.  Mirrors SetParametersNSsites (codeml.c:2381-2414,
// 2488-2521) and eigenQcodon / eigenQREV (codeml.c:3103-3273,
// tools.c:4850-4937) in the library's own code.
#pragma once

#include <cstdint>

namespace gb {

constexpr int NC = 61;

struct ModelParams {
    double kappa, w0, w2, p0, p1;
    double w1 = 1.0;         // site class 1's omega: 1 under model A, free under model B
    bool free_w1 = false;    // branch-site model B: w1 is a parameter (its derivatives are kept)
};

struct Derived {
    // eigen solutions for w0, w1 = 1, w2: Q_i = U_i diag(Root_i) V_i, row-major 61x61
    double U[3][NC * NC], V[3][NC * NC], Root[3][NC];
    double qf[2];        // Qfactor_NS_branch: background, foreground
    double freqK[4];     // p0, p1, p2a, p2b
    int sym = 1;         // V[m][k] = U[k][m] pi_k (true for eigen_qrev's solutions)
    // derivatives (filled when requested)
    double dqf[2][6];    // d qf[b] / d (kappa, w0, w2, p0, p1, w1)
    double dfreqK[4][2]; // d freqK[c] / d (p0, p1)
    double dQk[3][NC * NC];  // dQ_i/dkappa (row-major)
    double dQw[3][NC * NC];  // dQ_i/dw_i (zero matrix for w1 = 1)
};

// GY94 Q for (kappa, omega) with codon frequencies pi; returns the mean rate
// -sum_i pi_i Q_ii.  dQk/dQw (nullable) receive dQ/dkappa and dQ/domega.
double build_q(const double *pi, double kappa, double omega, double *Q, double *dQk, double *dQw);

// GY94's mean rate as part[0] + kappa part[1] + omega part[2] + kappa omega part[3]
void mean_rate_parts(const double *pi, double part[4]);

// Symmetric eigen solution of a reversible Q: Q = U diag(Root) V, V = U^-1.
// Householder tridiagonalisation (column-wise reflectors, Golub & Van Loan
// alg. 8.3.1) + implicit QL.  Returns 0 or -1 (no convergence).
int eigen_qrev(const double *Q, const double *pi, double *U, double *V, double *Root);

// Fill everything a model-A evaluation needs; 0 or GB_ERR_PARAM.
int derive(const double *pi, const ModelParams &m, bool want_grad, Derived *out, bool threads = true);

// Only the parts that do not need an eigen solution (Qfactors, freqK and
// their derivatives), for evaluations that receive U, V, Root from the host.
int derive_scalars(const double *pi, const ModelParams &m, Derived *out);

}  // namespace gb
