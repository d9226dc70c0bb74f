// Host-side model A set-up (see model.h).
#include "model.h"

#include <cmath>
#include <cstring>
#include <thread>

#include "gbcodeml.h"

namespace gb {

namespace {

const char kAA64[] = "FFLLSSSSYY**CC*WLLLLPPPPHHQQRRRRIIIMTTTTNNKKSSRRVVVVAAAADDEEGGGG";

struct CodeTables {
    int sense[NC];
    // per ordered pair (i, j), i != j, differing at one position:
    // kind bit 1 = transition, bit 2 = nonsynonymous; -1 = not a single change
    signed char kind[NC * NC];
    CodeTables() {
        int n = 0;
        for (int i = 0; i < 64; i++)
            if (kAA64[i] != '*') sense[n++] = i;
        for (int i = 0; i < NC; i++)
            for (int j = 0; j < NC; j++) {
                kind[i * NC + j] = -1;
                if (i == j) continue;
                int a = sense[i], b = sense[j];
                int fa[3] = {a / 16, (a / 4) % 4, a % 4}, fb[3] = {b / 16, (b / 4) % 4, b % 4};
                int nd = 0, pos = 0;
                for (int k = 0; k < 3; k++)
                    if (fa[k] != fb[k]) { nd++; pos = k; }
                if (nd != 1) continue;
                int s = fa[pos] + fb[pos];
                int ts = (s == 1 || s == 5);          // T<->C or A<->G
                int nsy = kAA64[a] != kAA64[b];
                kind[i * NC + j] = (signed char)(ts | (nsy << 1));
            }
    }
};

const CodeTables &tables() {
    static CodeTables t;
    return t;
}

// Householder reduction of the symmetric matrix a (row-major, n x n) to
// tridiagonal form.  On return a holds the accumulated orthogonal transform,
// d the diagonal and e[1..n-1] the sub-diagonal (e[0] = 0).
void householder_tridiag(int n, double *a, double *d, double *e) {
    for (int i = n - 1; i > 0; i--) {
        int l = i - 1;
        double h = 0;
        if (l > 0) {
            double scale = 0;
            for (int k = 0; k <= l; k++) scale += std::fabs(a[i * n + k]);
            if (scale == 0.0) {
                e[i] = a[i * n + l];
            } else {
                for (int k = 0; k <= l; k++) {
                    a[i * n + k] /= scale;
                    h += a[i * n + k] * a[i * n + k];
                }
                double f = a[i * n + l];
                double g = f >= 0 ? -std::sqrt(h) : std::sqrt(h);
                e[i] = scale * g;
                h -= f * g;
                a[i * n + l] = f - g;
                f = 0;
                for (int j = 0; j <= l; j++) {
                    a[j * n + i] = a[i * n + j] / h;
                    double gg = 0;
                    for (int k = 0; k <= j; k++) gg += a[j * n + k] * a[i * n + k];
                    for (int k = j + 1; k <= l; k++) gg += a[k * n + j] * a[i * n + k];
                    e[j] = gg / h;
                    f += e[j] * a[i * n + j];
                }
                double hh = f / (h + h);
                for (int j = 0; j <= l; j++) {
                    double ff = a[i * n + j];
                    double gg = e[j] - hh * ff;
                    e[j] = gg;
                    for (int k = 0; k <= j; k++) a[j * n + k] -= ff * e[k] + gg * a[i * n + k];
                }
            }
        } else {
            e[i] = a[i * n + l];
        }
        d[i] = h;
    }
    d[0] = 0;
    e[0] = 0;
    for (int i = 0; i < n; i++) {
        int l = i - 1;
        if (d[i] != 0.0) {
            for (int j = 0; j <= l; j++) {
                double g = 0;
                for (int k = 0; k <= l; k++) g += a[i * n + k] * a[k * n + j];
                for (int k = 0; k <= l; k++) a[k * n + j] -= g * a[k * n + i];
            }
        }
        d[i] = a[i * n + i];
        a[i * n + i] = 1;
        for (int j = 0; j <= l; j++) a[j * n + i] = a[i * n + j] = 0;
    }
}

// Implicit-shift QL on the tridiagonal (d, e); z accumulates the rotations
// (eigenvectors in columns).  Returns 0, or -1 if an eigenvalue did not
// converge in 60 iterations.
int ql_implicit(int n, double *d, double *e, double *z) {
    for (int i = 1; i < n; i++) e[i - 1] = e[i];
    e[n - 1] = 0;
    for (int l = 0; l < n; l++) {
        int iter = 0, m;
        do {
            for (m = l; m < n - 1; m++) {
                double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(e[m]) <= 1e-16 * dd) break;
            }
            if (m != l) {
                if (iter++ == 60) return -1;
                double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
                double r = std::hypot(g, 1.0);
                g = d[m] - d[l] + e[l] / (g + std::copysign(r, g));
                double s = 1, c = 1, p = 0;
                int i;
                bool underflow = false;
                for (i = m - 1; i >= l; i--) {
                    double f = s * e[i], b = c * e[i];
                    r = std::hypot(f, g);
                    e[i + 1] = r;
                    if (r == 0.0) {
                        d[i + 1] -= p;
                        e[m] = 0;
                        underflow = true;
                        break;
                    }
                    s = f / r;
                    c = g / r;
                    g = d[i + 1] - p;
                    r = (d[i] - g) * s + 2.0 * c * b;
                    p = s * r;
                    d[i + 1] = g + p;
                    g = c * r - b;
                    for (int k = 0; k < n; k++) {
                        double zf = z[k * n + i + 1];
                        z[k * n + i + 1] = s * z[k * n + i] + c * zf;
                        z[k * n + i] = c * z[k * n + i] - s * zf;
                    }
                }
                if (underflow) continue;
                d[l] -= p;
                e[l] = g;
                e[m] = 0;
            }
        } while (m != l);
    }
    return 0;
}

double mean_rate_omega(const double *pi, double kappa, double omega) {
    double Q[NC * NC];
    return build_q(pi, kappa, omega, Q, nullptr, nullptr);
}

// mean rate of GY94 as A + kappa B + omega C + kappa omega D
void rate_parts(const double *pi, double part[4]) {
    const CodeTables &T = tables();
    part[0] = part[1] = part[2] = part[3] = 0;
    for (int i = 0; i < NC; i++)
        for (int j = 0; j < NC; j++) {
            int k = T.kind[i * NC + j];
            if (k < 0) continue;
            part[k] += pi[i] * pi[j];
        }
}

}  // namespace

double build_q(const double *pi, double kappa, double omega, double *Q, double *dQk, double *dQw) {
    const CodeTables &T = tables();
    for (int i = 0; i < NC * NC; i++) Q[i] = 0;
    if (dQk) std::memset(dQk, 0, sizeof(double) * NC * NC);
    if (dQw) std::memset(dQw, 0, sizeof(double) * NC * NC);
    for (int i = 0; i < NC; i++)
        for (int j = 0; j < NC; j++) {
            int k = T.kind[i * NC + j];
            if (k < 0) continue;
            double q = (k & 1) ? kappa : 1.0;
            if (k & 2) q *= omega;
            Q[i * NC + j] = q * pi[j];
            if (dQk && (k & 1)) dQk[i * NC + j] = ((k & 2) ? omega : 1.0) * pi[j];
            if (dQw && (k & 2)) dQw[i * NC + j] = ((k & 1) ? kappa : 1.0) * pi[j];
        }
    double mr = 0;
    for (int i = 0; i < NC; i++) {
        double s = 0, sk = 0, sw = 0;
        for (int j = 0; j < NC; j++) {
            s += Q[i * NC + j];
            if (dQk) sk += dQk[i * NC + j];
            if (dQw) sw += dQw[i * NC + j];
        }
        Q[i * NC + i] = -s;
        if (dQk) dQk[i * NC + i] = -sk;
        if (dQw) dQw[i * NC + i] = -sw;
    }
    for (int i = 0; i < NC; i++) mr -= pi[i] * Q[i * NC + i];
    return mr;
}

int eigen_qrev(const double *Q, const double *pi, double *U, double *V, double *Root) {
    double a[NC * NC], e[NC], sq[NC];
    for (int i = 0; i < NC; i++) {
        if (!(pi[i] > 0)) return -1;
        sq[i] = std::sqrt(pi[i]);
    }
    for (int i = 0; i < NC; i++) {
        a[i * NC + i] = Q[i * NC + i];
        for (int j = 0; j < i; j++) a[i * NC + j] = a[j * NC + i] = Q[i * NC + j] * sq[i] / sq[j];
    }
    householder_tridiag(NC, a, Root, e);
    if (ql_implicit(NC, Root, e, a)) return -1;
    for (int i = 0; i < NC; i++)
        for (int k = 0; k < NC; k++) {
            U[i * NC + k] = a[i * NC + k] / sq[i];
            V[k * NC + i] = a[i * NC + k] * sq[i];
        }
    return 0;
}

int derive_scalars(const double *pi, const ModelParams &m, Derived *out) {
    double s = m.p0 + m.p1;
    if (!(s >= 1e-100) || !(m.p0 >= 0) || !(m.p1 >= 0) || !(s <= 1.0 + 1e-12) || !(m.kappa > 0) ||
        !(m.w0 >= 0) || !(m.w2 >= 0))
        return GB_ERR_PARAM;
    out->freqK[0] = m.p0;
    out->freqK[1] = m.p1;
    out->freqK[2] = (1 - s) * m.p0 / s;
    out->freqK[3] = (1 - s) * m.p1 / s;
    // Qfactor_NS_branch: background mixes (w0, 1) by p/(p0+p1); foreground (w0, 1, w2) by (p0, p1, 1-s)
    double wb = m.p0 / s * m.w0 + m.p1 / s * 1.0;
    double wf = m.p0 * m.w0 + m.p1 * 1.0 + (1 - s) * m.w2;
    double mr[2] = {mean_rate_omega(pi, m.kappa, wb), mean_rate_omega(pi, m.kappa, wf)};
    out->qf[0] = 1 / mr[0];
    out->qf[1] = 1 / mr[1];

    double part[4];
    rate_parts(pi, part);
    double wbar[2] = {wb, wf};
    // d wbar / d (w0, w2, p0, p1)
    double dw[2][4] = {
        {m.p0 / s, 0, m.p1 * (m.w0 - 1) / (s * s), m.p0 * (1 - m.w0) / (s * s)},
        {m.p0, 1 - s, m.w0 - m.w2, 1 - m.w2},
    };
    for (int b = 0; b < 2; b++) {
        double q2 = -out->qf[b] * out->qf[b];
        double dmr_dk = part[1] + wbar[b] * part[3];
        double dmr_dw = part[2] + m.kappa * part[3];
        out->dqf[b][0] = q2 * dmr_dk;
        for (int t = 0; t < 4; t++) out->dqf[b][1 + t] = q2 * dmr_dw * dw[b][t];
    }
    double s2 = s * s;
    out->dfreqK[0][0] = 1; out->dfreqK[0][1] = 0;
    out->dfreqK[1][0] = 0; out->dfreqK[1][1] = 1;
    out->dfreqK[2][0] = m.p1 / s2 - 1; out->dfreqK[2][1] = -m.p0 / s2;
    out->dfreqK[3][0] = -m.p1 / s2;    out->dfreqK[3][1] = m.p0 / s2 - 1;
    return 0;
}

int derive(const double *pi, const ModelParams &m, bool want_grad, Derived *out, bool threads) {
    int rc = derive_scalars(pi, m, out);
    if (rc) return rc;
    const double w[3] = {m.w0, 1.0, m.w2};
    int status[3] = {0, 0, 0};
    auto one = [&](int i) {
        double Q[NC * NC];
        build_q(pi, m.kappa, w[i], Q, want_grad ? out->dQk[i] : nullptr,
                want_grad ? out->dQw[i] : nullptr);
        status[i] = eigen_qrev(Q, pi, out->U[i], out->V[i], out->Root[i]);
        if (want_grad && i == 1) std::memset(out->dQw[1], 0, sizeof(double) * NC * NC);
    };
    // the three eigen problems are independent: side by side for a single
    // alignment; one after the other when the caller is already parallel
    // over alignments (a batch)
    if (threads) {
        std::thread t1(one, 1), t2(one, 2);
        one(0);
        t1.join();
        t2.join();
    } else {
        for (int i = 0; i < 3; i++) one(i);
    }
    for (int i = 0; i < 3; i++)
        if (status[i]) return GB_ERR_PARAM;
    return 0;
}

}  // namespace gb
