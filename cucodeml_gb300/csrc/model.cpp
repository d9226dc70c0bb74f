// Host-side model A set-up (see model.h).
#include "model.h"

#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
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

// Reduction of a symmetric matrix to tridiagonal form by Householder
// reflectors, column by column from the left (Golub & Van Loan, "Matrix
// Computations", 4th ed., algorithm 8.3.1; the same scheme as LAPACK's
// dsytd2 on the lower triangle followed by dorgtr).
//
// a: row-major n x n, full symmetric storage; overwritten.  Step k builds
// H_k = I - tau_k v v^T, v = (1, v_1, .., v_{m-1}) over rows k+1..n-1, that
// maps the column below the diagonal onto its first entry, and applies it to
// the trailing block in the symmetric rank-2 form S <- S - v w^T - w v^T with
// p = tau S v, w = p - (tau / 2)(p . v) v.  v_1.. are kept in column k under
// the sub-diagonal.  On return d holds the diagonal, e[k] the entry that
// couples k and k+1 (e[n-1] = 0), and qt the transpose of q = H_0 H_1 ..
// H_{n-3} (row-major), accumulated backwards, so that a_in = q T q^T.
void tridiagonalize(int n, double *a, double *d, double *e, double *qt) {
    double tau[NC], v[NC], p[NC];
    for (int k = 0; k + 2 < n; k++) {
        const int m = n - k - 1;
        double *S = a + (size_t)(k + 1) * n + (k + 1);      // S[r * n + c], r, c < m
        auto x = [&](int i) -> double & { return a[(size_t)(k + 1 + i) * n + k]; };
        d[k] = a[(size_t)k * n + k];
        const double alpha = x(0);
        double big = 0;
        for (int i = 1; i < m; i++) big = std::fmax(big, std::fabs(x(i)));
        if (big == 0.0) {                                    // already reduced
            tau[k] = 0;
            e[k] = alpha;
            continue;
        }
        double ss = 0;
        for (int i = 1; i < m; i++) {
            const double t = x(i) / big;
            ss += t * t;
        }
        const double beta = -std::copysign(std::hypot(alpha, big * std::sqrt(ss)), alpha);
        tau[k] = (beta - alpha) / beta;
        const double inv = 1.0 / (alpha - beta);
        v[0] = 1.0;
        for (int i = 1; i < m; i++) v[i] = (x(i) *= inv);
        e[k] = beta;
        double pv = 0;
        for (int r = 0; r < m; r++) {
            double s = 0;
            for (int c = 0; c < m; c++) s += S[(size_t)r * n + c] * v[c];
            p[r] = tau[k] * s;
            pv += p[r] * v[r];
        }
        const double half = 0.5 * tau[k] * pv;
        for (int r = 0; r < m; r++) p[r] -= half * v[r];           // p is now w
        for (int r = 0; r < m; r++)
            for (int c = 0; c < m; c++) S[(size_t)r * n + c] -= v[r] * p[c] + p[r] * v[c];
    }
    d[n - 2] = a[(size_t)(n - 2) * n + (n - 2)];
    e[n - 2] = a[(size_t)(n - 1) * n + (n - 2)];
    d[n - 1] = a[(size_t)(n - 1) * n + (n - 1)];
    e[n - 1] = 0;
    // q^T, accumulated backwards: q^T <- q^T H_k on columns k+1.. (rows of q^T
    // are the columns of q, contiguous)
    for (int i = 0; i < n * n; i++) qt[i] = 0;
    for (int i = 0; i < n; i++) qt[(size_t)i * n + i] = 1;
    for (int k = n - 3; k >= 0; k--) {
        if (tau[k] == 0.0) continue;
        const int m = n - k - 1;
        v[0] = 1.0;
        for (int i = 1; i < m; i++) v[i] = a[(size_t)(k + 1 + i) * n + k];
        for (int c = k + 1; c < n; c++) {
            double *__restrict__ row = qt + (size_t)c * n + (k + 1);
            double s = 0;
            for (int r = 0; r < m; r++) s += v[r] * row[r];
            s *= tau[k];
            for (int r = 0; r < m; r++) row[r] -= s * v[r];
        }
    }
}

// sqrt(a^2 + b^2): the plain form when the sum of squares is comfortably
// inside the double range (always, for rate matrices), std::hypot otherwise;
// the plain form is about twice as fast and within an ulp
inline double norm2(double a, double b) {
    const double s = a * a + b * b;
    return (s > 1e-290 && s < 1e290) ? std::sqrt(s) : std::hypot(a, b);
}

// Implicit-shift QL on the tridiagonal (d, e), e[k] coupling k and k+1.
// zt holds the transform transposed (row i = column i of the matrix the
// rotations multiply from the right), so that each rotation combines two
// contiguous rows; on return row i of zt is the eigenvector of d[i].  Returns
// 0, or -1 if an eigenvalue did not converge in 60 iterations.
int ql_implicit(int n, double *d, double *e, double *zt) {
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
                double r = norm2(g, 1.0);
                g = d[m] - d[l] + e[l] / (g + std::copysign(r, g));
                double s = 1, c = 1, p = 0;
                int i;
                bool underflow = false;
                for (i = m - 1; i >= l; i--) {
                    double f = s * e[i], b = c * e[i];
                    r = norm2(f, g);
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
                    double *__restrict__ za = zt + (size_t)i * n;
                    double *__restrict__ zb = zt + (size_t)(i + 1) * n;
                    for (int k = 0; k < n; k++) {
                        const double zf = zb[k];
                        zb[k] = s * za[k] + c * zf;
                        za[k] = c * za[k] - s * zf;
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

// Two long-lived helper threads for the side-by-side eigen solutions of one
// evaluation (starting threads per evaluation costs about as much as a
// 61 x 61 eigen solution).  One caller at a time: a caller that finds the
// helpers busy (another host thread's evaluation) runs its jobs itself.
class Helpers {
  public:
    static Helpers &get() {     // never destroyed: its threads live until the process exits
        static Helpers *h = new Helpers;
        return *h;
    }
    // job(1) and job(2) on the helpers, job(0) on the caller; false if busy
    bool run3(const std::function<void(int)> &job) {
        std::unique_lock<std::mutex> use(use_, std::try_to_lock);
        if (!use.owns_lock()) return false;
        {
            std::lock_guard<std::mutex> lk(mu_);
            job_ = &job;
            left_ = 2;
            gen_++;
        }
        cv_.notify_all();
        job(0);
        std::unique_lock<std::mutex> lk(mu_);
        done_.wait(lk, [&] { return left_ == 0; });
        job_ = nullptr;
        return true;
    }

  private:
    Helpers() {
        for (int w = 1; w <= 2; w++) std::thread([this, w] { loop(w); }).detach();
    }
    void loop(int w) {
        unsigned long seen = 0;
        for (;;) {
            const std::function<void(int)> *job;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                job = job_;
            }
            (*job)(w);
            std::lock_guard<std::mutex> lk(mu_);
            if (--left_ == 0) done_.notify_one();
        }
    }
    std::mutex use_, mu_;
    std::condition_variable cv_, done_;
    const std::function<void(int)> *job_ = nullptr;
    unsigned long gen_ = 0;
    int left_ = 0;
};

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

void mean_rate_parts(const double *pi, double part[4]) { rate_parts(pi, part); }

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
    double a[NC * NC], z[NC * NC], e[NC], sq[NC];
    for (int i = 0; i < NC; i++) {
        if (!(pi[i] > 0)) return -1;
        sq[i] = std::sqrt(pi[i]);
    }
    for (int i = 0; i < NC; i++) {
        a[i * NC + i] = Q[i * NC + i];
        for (int j = 0; j < i; j++) a[i * NC + j] = a[j * NC + i] = Q[i * NC + j] * sq[i] / sq[j];
    }
    tridiagonalize(NC, a, Root, e, z);
    if (ql_implicit(NC, Root, e, z)) return -1;
    // z row k = eigenvector k: U[i][k] = z[k][i] / sqrt(pi_i), V[k][i] = z[k][i] sqrt(pi_i)
    for (int k = 0; k < NC; k++)
        for (int i = 0; i < NC; i++) {
            U[i * NC + k] = z[k * NC + i] / sq[i];
            V[k * NC + i] = z[k * NC + i] * sq[i];
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
    // Qfactor_NS_branch: background mixes (w0, w1) by p/(p0+p1); foreground (w0, w1, w2) by
    // (p0, p1, 1-s); w1 = 1 under model A
    const double w1 = m.w1;
    if (!(w1 >= 0)) return GB_ERR_PARAM;
    double wb = m.p0 / s * m.w0 + m.p1 / s * w1;
    double wf = m.p0 * m.w0 + m.p1 * w1 + (1 - s) * m.w2;
    double mr[2] = {mean_rate_omega(pi, m.kappa, wb), mean_rate_omega(pi, m.kappa, wf)};
    out->qf[0] = 1 / mr[0];
    out->qf[1] = 1 / mr[1];

    double part[4];
    rate_parts(pi, part);
    double wbar[2] = {wb, wf};
    // d wbar / d (w0, w2, p0, p1, w1)
    double dw[2][5] = {
        {m.p0 / s, 0, m.p1 * (m.w0 - w1) / (s * s), m.p0 * (w1 - m.w0) / (s * s), m.p1 / s},
        {m.p0, 1 - s, m.w0 - m.w2, w1 - m.w2, m.p1},
    };
    for (int b = 0; b < 2; b++) {
        double q2 = -out->qf[b] * out->qf[b];
        double dmr_dk = part[1] + wbar[b] * part[3];
        double dmr_dw = part[2] + m.kappa * part[3];
        out->dqf[b][0] = q2 * dmr_dk;
        for (int t = 0; t < 5; t++) out->dqf[b][1 + t] = q2 * dmr_dw * dw[b][t];
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
    const double w[3] = {m.w0, m.w1, m.w2};
    int status[3] = {0, 0, 0};
    auto one = [&](int i) {
        double Q[NC * NC];
        build_q(pi, m.kappa, w[i], Q, want_grad ? out->dQk[i] : nullptr,
                want_grad ? out->dQw[i] : nullptr);
        status[i] = eigen_qrev(Q, pi, out->U[i], out->V[i], out->Root[i]);
        if (want_grad && i == 1 && !m.free_w1) std::memset(out->dQw[1], 0, sizeof(double) * NC * NC);
    };
    // the three eigen problems are independent: side by side for a single
    // alignment; one after the other when the caller is already parallel
    // over alignments (a batch)
    const std::function<void(int)> job = one;
    if (!threads || !Helpers::get().run3(job))
        for (int i = 0; i < 3; i++) one(i);
    for (int i = 0; i < 3; i++)
        if (status[i]) return GB_ERR_PARAM;
    return 0;
}

}  // namespace gb
