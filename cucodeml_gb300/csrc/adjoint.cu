// FP64 adjoint (reverse-mode) gradient of lnL for branch-site model A.
//
// The reference has no analytic gradient: codeml's optimiser ming2 takes a
// gradient hook (tools.c:6361-6363) but is given NULL (codeml.c:688), so every
// gradient costs np or 2np likelihood evaluations through gradientB
// (tools.c:6326-6350).  This module differentiates the forward evaluation of
// runtime.cu exactly:
//
//   forward  L_a = prod_i E_i,  E_i = P_i L~_{s_i}  (tips: rows of P),
//            L~_a = L_a / m_a at scaled nodes, f~ = pi . L~_root,
//            lnL = sum_h fpatt_h log sum_c freqK_c e^{S_c} f~_c.
//   seeds    dlnL/dL~_root,c[h][j] = fpatt_h rho_c,h / f~_c,h * pi_j
//            (rho = posterior of the site class).  Node scales m are held
//            constant: lnL is invariant to them.
//   sweep    top-down over the same levels: Ebar_i = (Abar_a / m_a) . prod_{i'!=i} E_i',
//            Abar_{s_i} += Ebar_i P_i, and dlnL/dP_i += sum_h Ebar_i[h]^T L~_{s_i}[h].
//            A child slot shared by two parent classes (class 2a = class 0 below
//            the foreground path) accumulates both contributions.
//   params   P = U e^{t' Root} V: dlnL/dt' = sum_m Root_m e^{t' Root_m} (U^T G V^T)_mm;
//            kappa / omega through dP = U [(V dQ U) o Phi] V t' with
//            Phi_mn = (e^{a_m} - e^{a_n}) / (a_m - a_n), a = t' Root;
//            Qfactors, class proportions and branch lengths by the chain rule
//            on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "handle.h"
#include "adjoint_internal.h"
#include "fast_device.cuh"
#include "batch_internal.h"

namespace gb {

namespace {

constexpr int NCd = 61;
constexpr int kGradPSmem = (2 * TILE64 * 65 + 64 * 65) * sizeof(double);
constexpr int kGradHSmem = (2 * 61 * 62 + 3 * 256 + 64) * sizeof(double);

// ---------------------------------------------------------------- kernels

// D matrices V dQ U for (kappa: w=0,1,2) and (omega: w=0,2 and slot 1), 64-padded,
// and the inverse eigenvalue differences of each w (for Phi)
// Block bid: derivative d = bid / DM_RB (0,1,2: kappa for w; 3: omega w0; 4:
// omega w2; 5: omega of slot 1, stored at DM_OMEGA1), output rows
// 16 (bid % DM_RB) .. + 15 of D = V dQ U; the last 3 blocks:
// 1/(Root_m - Root_n) for w (and U, V^T as double-float).
// dQ has at most ~10 non-zeros per row (single-nucleotide neighbours and the
// diagonal): T = dQ U runs over each row's non-zeros (dense past 16).
__device__ __forceinline__ float2 df_of(double v) {
    const float hi = (float)v;
    return make_float2(hi, (float)(v - (double)hi));
}

__device__ __forceinline__ void dmat_body(const DevParams *__restrict__ prm, const GradParams *__restrict__ gp,
                                          double *__restrict__ Dm, float2 *__restrict__ UVdf, int bid) {
    __shared__ double T[61 * 62];
    __shared__ int nzk[61][16];
    __shared__ double nzv[61][16];
    __shared__ int nnz[61];
    if (bid >= DM_NDER * DM_RB) {
        const int w = bid - DM_NDER * DM_RB, which = 5 + w;
        const double *R = prm->Root[w];
        double *out = Dm + (size_t)which * 64 * 64;
        for (int i = threadIdx.x; i < 64 * 64; i += blockDim.x) {
            const int r = i / 64, c = i % 64;
            const double d = (r < 61 && c < 61) ? R[r] - R[c] : 0.0;
            out[i] = d != 0.0 ? 1.0 / d : 0.0;
            if (UVdf) UVdf[UVDF_DM + (size_t)which * 64 * 64 + i] = df_of(out[i]);
        }
        if (UVdf) {   // V^T [k][n] and U [j][m] of this w as double-float, 64-column rows
            float2 *vt = UVdf + (size_t)w * 2 * 61 * 64, *u = vt + 61 * 64;
            for (int i = threadIdx.x; i < 61 * 64; i += blockDim.x) {
                const int r = i / 64, c = i % 64;
                const double a = c < 61 ? prm->V[w][c * 61 + r] : 0.0;
                const double b = c < 61 ? prm->U[w][r * 61 + c] : 0.0;
                const float ah = (float)a, bh = (float)b;
                vt[i] = make_float2(ah, (float)(a - (double)ah));
                u[i] = make_float2(bh, (float)(b - (double)bh));
            }
        }
        return;
    }
    const int d = bid / DM_RB, rb = bid % DM_RB;
    const int w = d < 3 ? d : (d == 3 ? 0 : (d == 4 ? 2 : 1));
    const int which = d == 5 ? DM_OMEGA1 : d;
    const double *dQ = d < 3 ? gp->dQk[w] : gp->dQw[w];
    const double *U = prm->U[w];
    const double *V = prm->V[w];
    if (threadIdx.x < 61) {               // non-zeros of row r of dQ
        const int r = threadIdx.x;
        int n = 0;
        for (int c = 0; c < 61; c++) {
            const double v = dQ[r * 61 + c];
            if (v != 0.0) {
                if (n < 16) {
                    nzk[r][n] = c;
                    nzv[r][n] = v;
                }
                n++;
            }
        }
        nnz[r] = n;
    }
    __syncthreads();
    // T = dQ U
    for (int i = threadIdx.x; i < 61 * 61; i += blockDim.x) {
        const int r = i / 61, c = i % 61;
        double s = 0;
        if (nnz[r] <= 16) {
            for (int q = 0; q < nnz[r]; q++) s = fma(nzv[r][q], U[nzk[r][q] * 61 + c], s);
        } else {
            for (int kk = 0; kk < 61; kk++) s = fma(dQ[r * 61 + kk], U[kk * 61 + c], s);
        }
        T[r * 62 + c] = s;
    }
    __syncthreads();
    double *out = Dm + (size_t)which * 64 * 64;
    const int r0 = rb * (64 / DM_RB);
    for (int i = threadIdx.x; i < (64 / DM_RB) * 64; i += blockDim.x) {
        const int r = r0 + i / 64, c = i % 64;
        double s = 0;
        if (r < 61 && c < 61)
            for (int kk = 0; kk < 61; kk++) s = fma(V[r * 61 + kk], T[kk * 62 + c], s);
        out[r * 64 + c] = s;
        if (UVdf) UVdf[UVDF_DM + (size_t)which * 64 * 64 + r * 64 + c] = df_of(s);
    }
}

__global__ void __launch_bounds__(256) dmat_kernel(const DevParams *__restrict__ prm,
                                                   const GradParams *__restrict__ gp,
                                                   double *__restrict__ Dm, float2 *__restrict__ UVdf) {
    dmat_body(prm, gp, Dm, UVdf, blockIdx.x);
}

__global__ void __launch_bounds__(256) dmat_batched_kernel(const DmatArgs *__restrict__ args,
                                                           const int2 *__restrict__ map) {
    const int2 g = map[blockIdx.x];
    const DmatArgs &a = args[g.x];
    dmat_body(a.prm, a.gp, a.Dm, a.UVdf, g.y);
}

// one CTA per (32-pattern tile, backward item)
__global__ void __launch_bounds__(128) bwd_level_kernel(
    const BItem *__restrict__ bitems, int npad, const double *__restrict__ Pt,
    const double *__restrict__ E, double *__restrict__ Ebar, double *__restrict__ Abar,
    const double *__restrict__ scaleF, const double *__restrict__ fpatt,
    const double *__restrict__ post, const double *__restrict__ fbar, const double *__restrict__ pi) {
    __shared__ double Bs[NCd * 65];  // P[j][k] (non-transposed), rows j < 61
    __shared__ double Xs[TILE64 * 65];
    const BItem it = bitems[blockIdx.y];
    const int h0 = blockIdx.x * TILE64;
    const int tid = threadIdx.x;
    const int rg = tid >> 4, cg = tid & 15;
    const int r0 = rg * 4, c0 = cg * 4;

    double A[2][4][4];
    for (int k = 0; k < it.ncls; k++) {
        const int c = it.cls[k];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            const int h = h0 + r0 + r;
            double sc = 1.0;
            if (it.sslot[k] >= 0) {
                const double sf = scaleF[(size_t)it.sslot[k] * npad + h];
                sc = sf == -800.0 ? 0.0 : exp(-sf);
            }
            if (it.is_root) {
                const double g = fpatt[h] * post[(size_t)c * npad + h] / fbar[(size_t)c * npad + h];
#pragma unroll
                for (int q = 0; q < 4; q++) A[k][r][q] = (c0 + q < NCd) ? g * pi[c0 + q] : 0.0;
            } else {
                const double4 v = *reinterpret_cast<const double4 *>(Abar + ((size_t)it.pslot[k] * npad + h) * 64 + c0);
                A[k][r][0] = v.x * sc; A[k][r][1] = v.y * sc; A[k][r][2] = v.z * sc; A[k][r][3] = v.w * sc;
            }
        }
    }

    for (int i = 0; i < it.nchild; i++) {
        double Eb[2][4][4];
        for (int k = 0; k < it.ncls; k++) {
#pragma unroll
            for (int r = 0; r < 4; r++)
#pragma unroll
                for (int q = 0; q < 4; q++) Eb[k][r][q] = A[k][r][q];
            for (int i2 = 0; i2 < it.nchild; i2++) {
                if (i2 == i) continue;
                const double *e = E + ((size_t)(it.eslot[k] + i2) * npad + h0 + r0) * 64 + c0;
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    const double4 v = *reinterpret_cast<const double4 *>(e + r * 64);
                    Eb[k][r][0] *= v.x; Eb[k][r][1] *= v.y; Eb[k][r][2] *= v.z; Eb[k][r][3] *= v.w;
                }
            }
            double *eb = Ebar + ((size_t)(it.eslot[k] + i) * npad + h0 + r0) * 64 + c0;
#pragma unroll
            for (int r = 0; r < 4; r++)
                *reinterpret_cast<double4 *>(eb + r * 64) = make_double4(Eb[k][r][0], Eb[k][r][1], Eb[k][r][2], Eb[k][r][3]);
        }
        if (it.tslot[i][0] < 0) continue;   // tip child: only dlnL/dP (gradP kernel)
        // adjoint of the child: one target if both classes share it, else one per class
        const bool shared = it.ncls == 1 || it.tslot[i][0] == it.tslot[i][1];
        const int ntarget = shared ? 1 : 2;
        for (int tg = 0; tg < ntarget; tg++) {
            double acc[4][4];
#pragma unroll
            for (int r = 0; r < 4; r++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[r][q] = 0.0;
            const int kbeg = shared ? 0 : tg, kend = shared ? it.ncls : tg + 1;
            for (int k = kbeg; k < kend; k++) {
                const double *P = Pt + (size_t)it.pidx[i][k] * 64 * 64;
                __syncthreads();
                for (int idx = tid; idx < 64 * 64; idx += 128) {
                    const int kk = idx >> 6, jj = idx & 63;   // Pt[kk][jj] = P[jj][kk]
                    if (jj < NCd) Bs[jj * 65 + kk] = P[idx];
                }
#pragma unroll
                for (int r = 0; r < 4; r++)
#pragma unroll
                    for (int q = 0; q < 4; q++) Xs[(r0 + r) * 65 + c0 + q] = Eb[k][r][q];
                __syncthreads();
#pragma unroll 4
                for (int j = 0; j < NCd; j++) {
                    double a[4], b[4];
#pragma unroll
                    for (int r = 0; r < 4; r++) a[r] = Xs[(r0 + r) * 65 + j];
#pragma unroll
                    for (int q = 0; q < 4; q++) b[q] = Bs[j * 65 + c0 + q];
#pragma unroll
                    for (int r = 0; r < 4; r++)
#pragma unroll
                        for (int q = 0; q < 4; q++) acc[r][q] = fma(a[r], b[q], acc[r][q]);
                }
            }
            double *o = Abar + ((size_t)it.tslot[i][tg] * npad + h0 + r0) * 64 + c0;
#pragma unroll
            for (int r = 0; r < 4; r++)
                *reinterpret_cast<double4 *>(o + r * 64) = make_double4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
        }
    }
}

// partial dlnL/dP of one pair over a chunk of patterns: G[j][k] = sum_h Ebar[h][j] X[h][k]
__global__ void __launch_bounds__(128) gradP_kernel(const Contrib *__restrict__ contrib,
                                                    const int *__restrict__ coff, int npatt, int npad,
                                                    const double *__restrict__ Ebar,
                                                    const double *__restrict__ conP,
                                                    const unsigned char *__restrict__ z,
                                                    double *__restrict__ Gpart, int nchunk,
                                                    const unsigned char *__restrict__ amb,
                                                    const int *__restrict__ plist) {
    extern __shared__ double smg[];
    double *Es = smg;                    // [32][65]
    double *Xs = smg + TILE64 * 65;      // [32][65]
    double *Gs = smg + 2 * TILE64 * 65;  // [64][65] tip scatter target
    const int p = plist ? plist[blockIdx.x] : (int)blockIdx.x, chunk = blockIdx.y;
    const int tid = threadIdx.x;
    // thread owns G rows j = 8*(tid/16) .. +7, cols k = 4*(tid%16) .. +3
    const int j0 = (tid >> 4) * 8, k0 = (tid & 15) * 4;
    double g[8][4];
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) g[a][b] = 0.0;
    for (int i = tid; i < 64 * 65; i += 128) Gs[i] = 0.0;
    const int hbeg = chunk * GCHUNK, hend = min(npatt, hbeg + GCHUNK);
    for (int ci = coff[p]; ci < coff[p + 1]; ci++) {
        const Contrib cb = contrib[ci];
        for (int hb = hbeg; hb < hend; hb += TILE64) {
            __syncthreads();
            const double *eb = Ebar + ((size_t)cb.ebar * npad + hb) * 64;
            for (int i = tid; i < TILE64 * 64; i += 128) Es[(i >> 6) * 65 + (i & 63)] = eb[i];
            if (cb.tslot >= 0) {
                const double *x = conP + ((size_t)cb.tslot * npad + hb) * 64;
                for (int i = tid; i < TILE64 * 64; i += 128) Xs[(i >> 6) * 65 + (i & 63)] = x[i];
            }
            __syncthreads();
            const int nh = min(TILE64, hend - hb);
            if (cb.tslot >= 0) {
                for (int hh = 0; hh < nh; hh++) {
                    double a[8], b[4];
#pragma unroll
                    for (int q = 0; q < 8; q++) a[q] = Es[hh * 65 + j0 + q];
#pragma unroll
                    for (int q = 0; q < 4; q++) b[q] = Xs[hh * 65 + k0 + q];
#pragma unroll
                    for (int q = 0; q < 8; q++)
#pragma unroll
                        for (int u = 0; u < 4; u++) g[q][u] = fma(a[q], b[u], g[q][u]);
                }
            } else if (tid < 64) {
                // tip: X is one-hot at z[h]; thread tid owns row j = tid of Gs
                const unsigned char *zz = z + (size_t)cb.tip * npad + hb;
                for (int hh = 0; hh < nh; hh++) {
                    const int c = zz[hh];
                    if (c < NCd || !amb) {
                        Gs[tid * 65 + c] += Es[hh * 65 + tid];
                    } else {   // ambiguous codon: X[h][k] = 1 for each sense codon k it stands for
                        const unsigned char *map = amb + 256 + 64 * c;
                        for (int q = 0; q < amb[c]; q++) Gs[tid * 65 + map[q]] += Es[hh * 65 + tid];
                    }
                }
            }
        }
    }
    __syncthreads();
    double *out = Gpart + ((size_t)p * nchunk + chunk) * 64 * 64;
#pragma unroll
    for (int q = 0; q < 8; q++)
#pragma unroll
        for (int u = 0; u < 4; u++) out[(j0 + q) * 64 + k0 + u] = g[q][u] + Gs[(j0 + q) * 65 + k0 + u];
}

// Phi_mn = (e^{a_m} - e^{a_n}) / (a_m - a_n), a = t' Root, from em = e^{a_m},
// en = e^{a_n} and inv = 1 / (Root_m - Root_n): the divided difference when
// |a_m - a_n| >= 1e-3 (relative error <= eps / 1e-3), else the series
// e^{(a_m + a_n)/2} (1 + d^2/24 + d^4/1920)
__device__ __forceinline__ double phi_of(double am, double an, double em, double en, double inv, double rtp) {
    const double d = am - an;
    if (fabs(d) < 1e-3) {
        const double d2 = d * d;
        return sqrt(em * en) * (1.0 + d2 * (1.0 / 24.0 + d2 * (1.0 / 1920.0)));
    }
    return (em - en) * inv * rtp;
}

// per pair: G = sum of chunk partials; H = U^T G V^T; contributions to dlnL/dt',
// dlnL/dkappa and dlnL/domega (out[pair][3])
__global__ void __launch_bounds__(256) gradH_kernel(const PairDesc *__restrict__ pairs,
                                                    const int *__restrict__ label,
                                                    const double *__restrict__ tnode,
                                                    const DevParams *__restrict__ prm,
                                                    const double *__restrict__ Gpart, int nchunk,
                                                    const double *__restrict__ Dm,
                                                    double *__restrict__ out) {
    extern __shared__ double smh[];
    double *Gs = smh;                    // [61][62]
    double *Ts = smh + 61 * 62;          // [61][62]
    double (*red)[256] = reinterpret_cast<double (*)[256]>(smh + 2 * 61 * 62);
    double *ex = smh + 2 * 61 * 62 + 3 * 256;   // [64] e^{t' Root_m}
    const int p = blockIdx.x;
    const PairDesc pd = pairs[p];
    const int w = pd.w;
    const double tp = tnode[pd.node] * prm->qf[label[pd.node]];
    const double *U = prm->U[w];
    const double *V = prm->V[w];
    const double *R = prm->Root[w];
    if (threadIdx.x < 61) ex[threadIdx.x] = exp(tp * R[threadIdx.x]);
    for (int i = threadIdx.x; i < 61 * 61; i += blockDim.x) {
        int j = i / 61, k = i % 61;
        double s = 0;
        for (int c = 0; c < nchunk; c++) s += Gpart[((size_t)p * nchunk + c) * 64 * 64 + j * 64 + k];
        Gs[j * 62 + k] = s;
    }
    __syncthreads();
    // T = G V^T : T[j][n] = sum_k G[j][k] V[n][k]
    for (int i = threadIdx.x; i < 61 * 61; i += blockDim.x) {
        int j = i / 61, n = i % 61;
        double s = 0;
        for (int k = 0; k < 61; k++) s = fma(Gs[j * 62 + k], V[n * 61 + k], s);
        Ts[j * 62 + n] = s;
    }
    __syncthreads();
    // H[m][n] = sum_j U[j][m] T[j][n]
    double sdt = 0, sk = 0, sw = 0;
    const double *Dk = Dm + (size_t)w * 64 * 64;
    const double *Dw = Dm + (size_t)(w == 0 ? 3 : (w == 2 ? 4 : DM_OMEGA1)) * 64 * 64;
    const double *inv = Dm + (size_t)(5 + w) * 64 * 64;
    const double rtp = tp > 0.0 ? 1.0 / tp : 0.0;
    for (int i = threadIdx.x; i < 61 * 61; i += blockDim.x) {
        int m = i / 61, n = i % 61;
        double hmn = 0;
        for (int j = 0; j < 61; j++) hmn = fma(U[j * 61 + m], Ts[j * 62 + n], hmn);
        const double phi = phi_of(tp * R[m], tp * R[n], ex[m], ex[n], inv[m * 64 + n], rtp);
        if (m == n) sdt += R[m] * ex[m] * hmn;
        const double hp = hmn * phi * tp;
        sk = fma(hp, Dk[m * 64 + n], sk);
        if (Dw) sw = fma(hp, Dw[m * 64 + n], sw);
    }
    red[0][threadIdx.x] = sdt;
    red[1][threadIdx.x] = sk;
    red[2][threadIdx.x] = sw;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 3; q++) red[q][threadIdx.x] += red[q][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 3) out[p * 3 + threadIdx.x] = red[threadIdx.x][0];
}

// The same per-pair sums for the split-precision path, with the two 61^3
// products in double-float on the FP32 pipe (no FP64 arithmetic in the
// contractions): every term's product error is recovered exactly with an FMA
// and the sums are compensated (TwoSum of the high parts, errors summed
// apart), then H is rounded to FP64 for the Phi-weighted sums.
// Thread (r = tid / 4, c0 = 16 (tid % 4)) owns row r, columns c0..c0+15.
__device__ __forceinline__ void dot2_step(float &s, float &c, float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    const float t = s + p;
    const float z = t - s;
    c += ((s - (t - z)) + (p - z)) + e;
    s = t;
}


constexpr int kGradHdfSmem = (61 * 66 + 2 * 61 * 64) * 8 + (64 + 3 * 256) * 8 + 2 * 64 * 8;

// Shared-memory layout: G (then T) rows padded to GS = 66 double-float so that
// the 8 rows a warp reads at one k fall in different banks; thread
// (r = tid / 4, q = tid % 4) owns row r and the interleaved columns q + 4 i,
// so the 4 column groups of a warp read 4 consecutive entries (no conflict).
constexpr int GS = 66;

__device__ __forceinline__ void gradH_df_body(const PairDesc *__restrict__ pairs, const int *__restrict__ label,
                                              const double *__restrict__ tnode, const DevParams *__restrict__ prm,
                                              const float2 *__restrict__ Gpart, int nchunk,
                                              const double *__restrict__ Dm, const float2 *__restrict__ UVdf,
                                              double *__restrict__ out, int p) {
    extern __shared__ __align__(16) unsigned char smr[];
    float2 *GT = reinterpret_cast<float2 *>(smr);          // [61][GS] G, then T
    float2 *Vt = GT + 61 * GS;                              // [61][64] Vt[k][n] = V[n][k]
    float2 *Us = Vt + 61 * 64;                              // [61][64] U[j][m]
    double *ex = reinterpret_cast<double *>(Us + 61 * 64);  // [64]
    double (*red)[256] = reinterpret_cast<double (*)[256]>(ex + 64);
    float2 *exd = reinterpret_cast<float2 *>(red[3]);       // [64] ex as double-float
    float2 *Rd = exd + 64;                                  // [64] Root as double-float
    const int tid = threadIdx.x;
    const PairDesc pd = pairs[p];
    const int w = pd.w;
    const double tp = tnode[pd.node] * prm->qf[label[pd.node]];
    const double *R = prm->Root[w];
    if (tid < 61) {
        ex[tid] = exp(tp * R[tid]);
        exd[tid] = df_of(ex[tid]);
        Rd[tid] = df_of(R[tid]);
    }
    {   // V^T and U of this w, already double-float (dP/dt kernel)
        const float4 *src = reinterpret_cast<const float4 *>(UVdf + (size_t)w * 2 * 61 * 64);
        float4 *dst = reinterpret_cast<float4 *>(Vt);
        for (int i = tid; i < 61 * 64; i += blockDim.x) dst[i] = src[i];
    }
    for (int i = tid; i < 61 * 64; i += blockDim.x) {      // G = sum of the chunk partials
        float2 g = make_float2(0.f, 0.f);
        for (int q = 0; q < nchunk; q++) g = fastdev::df_add(g, Gpart[((size_t)p * nchunk + q) * 64 * 64 + i]);
        GT[(i >> 6) * GS + (i & 63)] = (i & 63) < 61 ? g : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int r = tid >> 2, q4 = tid & 3;
    float s[16], e[16];
    // T[r][n] = sum_k G[r][k] Vt[k][n], n = q4 + 4 i
#pragma unroll
    for (int i = 0; i < 16; i++) s[i] = e[i] = 0.f;
    if (r < 61)
        for (int k = 0; k < 61; k++) {
            const float2 g = GT[r * GS + k];
#pragma unroll
            for (int i = 0; i < 16; i++) dot2_step(s[i], e[i], g, Vt[k * 64 + q4 + 4 * i]);
        }
    __syncthreads();                                        // every read of G is done
    if (r < 61)
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const float hi = s[i] + e[i];
            GT[r * GS + q4 + 4 * i] = make_float2(hi, e[i] - (hi - s[i]));
        }
    __syncthreads();
    // H[r][n] = sum_j U[j][r] T[j][n]
#pragma unroll
    for (int i = 0; i < 16; i++) s[i] = e[i] = 0.f;
    if (r < 61)
        for (int j = 0; j < 61; j++) {
            const float2 u = Us[j * 64 + r];
#pragma unroll
            for (int i = 0; i < 16; i++) dot2_step(s[i], e[i], u, GT[j * GS + q4 + 4 * i]);
        }
    // Phi-weighted sums in double-float on the FP32 pipe (the dP/dt and
    // inverse-difference tables in their double-float copies): with
    // d = t' (R_r - R_n), Phi = (e_r - e_n) inv_rn / t' except for |d| < 1e-3,
    // where the series of the FP64 path is used
    float2 sdt = make_float2(0.f, 0.f), sk = sdt, sw = sdt;
    const float2 *Tdf = UVdf + UVDF_DM;
    const float2 *Dk = Tdf + (size_t)w * 64 * 64;
    const float2 *Dw = Tdf + (size_t)(w == 0 ? 3 : (w == 2 ? 4 : DM_OMEGA1)) * 64 * 64;
    const float2 *inv = Tdf + (size_t)(5 + w) * 64 * 64;
    const double rtp = tp > 0.0 ? 1.0 / tp : 0.0;
    const float2 rtpd = df_of(rtp), tpd = df_of(tp);
    const float tpf = (float)tp;
    if (r < 61) {
        const float Rr = (float)R[r];
#pragma unroll
        for (int i = 0; i < 16; i++) {
            const int n = q4 + 4 * i;
            if (n >= 61) continue;
            const float2 hmn = fastdev::fast_two_sum(s[i], e[i]);
            float2 phi;
            if (fabsf(tpf * (Rr - (float)R[n])) < 1e-3f) {
                const double dd = tp * R[r] - tp * R[n], d2 = dd * dd;
                phi = df_of(sqrt(ex[r] * ex[n]) * (1.0 + d2 * (1.0 / 24.0 + d2 * (1.0 / 1920.0))));
            } else {
                const float2 de = fastdev::df_add(exd[r], make_float2(-exd[n].x, -exd[n].y));
                phi = fastdev::df_mul(fastdev::df_mul(de, inv[r * 64 + n]), rtpd);
            }
            if (r == n) sdt = fastdev::df_add(sdt, fastdev::df_mul(fastdev::df_mul(Rd[r], exd[r]), hmn));
            const float2 hp = fastdev::df_mul(fastdev::df_mul(hmn, phi), tpd);
            sk = fastdev::df_add(sk, fastdev::df_mul(hp, Dk[r * 64 + n]));
            if (Dw) sw = fastdev::df_add(sw, fastdev::df_mul(hp, Dw[r * 64 + n]));
        }
    }
    red[0][tid] = (double)sdt.x + (double)sdt.y;
    red[1][tid] = (double)sk.x + (double)sk.y;
    red[2][tid] = (double)sw.x + (double)sw.y;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (tid < st)
            for (int q = 0; q < 3; q++) red[q][tid] += red[q][tid + st];
        __syncthreads();
    }
    if (tid < 3) out[p * 3 + tid] = red[tid][0];
}

__global__ void __launch_bounds__(256) gradH_df_kernel(const PairDesc *__restrict__ pairs,
                                                       const int *__restrict__ label,
                                                       const double *__restrict__ tnode,
                                                       const DevParams *__restrict__ prm,
                                                       const float2 *__restrict__ Gpart, int nchunk,
                                                       const double *__restrict__ Dm,
                                                       const float2 *__restrict__ UVdf,
                                                       double *__restrict__ out) {
    gradH_df_body(pairs, label, tnode, prm, Gpart, nchunk, Dm, UVdf, out, blockIdx.x);
}

__global__ void __launch_bounds__(256) gradH_batched_kernel(const GradHArgs *__restrict__ args,
                                                            const int2 *__restrict__ map) {
    const int2 g = map[blockIdx.x];
    const GradHArgs &a = args[g.x];
    gradH_df_body(a.pairs, a.label, a.tnode, a.prm, a.Gpart, a.nchunk, a.Dm, a.UVdf, a.out, g.y);
}

// dlnL/dfreqK_c (up to the 1/freqK_c factor) : sum_h fpatt_h f_c / R_h
__device__ __forceinline__ void freq_body(const double *__restrict__ fhK, const double *__restrict__ lnf,
                                          const double *__restrict__ fpatt, int npatt, int npad, int nscale,
                                          double *__restrict__ part, int bid) {
    __shared__ double red[4][256];
    const int h = bid * blockDim.x + threadIdx.x;
    double q[4] = {0, 0, 0, 0};
    if (h < npatt && fpatt[h] > 0) {
        const double L = lnf[h];
        for (int c = 0; c < 4; c++) {
            const double v = fhK[(size_t)c * npad + h];
            q[c] = fpatt[h] * (nscale > 0 ? exp(v - L) : v / exp(L));
        }
    }
    for (int c = 0; c < 4; c++) red[c][threadIdx.x] = q[c];
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int c = 0; c < 4; c++) red[c][threadIdx.x] += red[c][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 4) part[bid * 4 + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void __launch_bounds__(256) freq_kernel(const double *__restrict__ fhK,
                                                   const double *__restrict__ lnf,
                                                   const double *__restrict__ fpatt, int npatt,
                                                   int npad, int nscale, double *__restrict__ part) {
    freq_body(fhK, lnf, fpatt, npatt, npad, nscale, part, blockIdx.x);
}

__global__ void __launch_bounds__(256) freq_batched_kernel(const FreqArgs *__restrict__ args,
                                                           const int2 *__restrict__ map) {
    const int2 g = map[blockIdx.x];
    const FreqArgs &a = args[g.x];
    freq_body(a.fhK, a.lnf, a.fpatt, a.npatt, a.npad, a.nscale, a.part, g.y);
}

}  // namespace



void adjoint_free(AdjointState *a) {
    if (!a) return;
    if (a->graph) cudaGraphExecDestroy(a->graph);
    void *dev[] = {a->d_bitems, a->d_contrib, a->d_coff, a->d_Ebar, a->d_Abar, a->d_Gpart,
                   a->d_Dm, a->d_pout, a->d_fpart, a->d_gp, a->d_UVdf, a->d_ritems, a->d_plist};
    for (void *p : dev)
        if (p) cudaFree(p);
    if (a->h_gp) cudaFreeHost(a->h_gp);
    if (a->h_pout) cudaFreeHost(a->h_pout);
    if (a->h_fpart) cudaFreeHost(a->h_fpart);
    delete a;
}

int adjoint_init(gb_handle *h) {
    if (h->adj) return 0;
    AdjointState *a = new AdjointState();
    h->adj = a;
    const int ns = h->ns, nn = h->nnode;
    auto ncls = [&](int n) { return (h->dirty[n] || n == h->root) ? 4 : 2; };
    auto cls_of = [&](int s, int c) { return (h->dirty[s] || s == h->root) ? c : (c & 1); };
    // backward items, levels from the root down
    const int H = h->height[h->root];
    a->blevel_off.clear();
    for (int L = H; L >= 1; L--) {
        a->blevel_off.push_back((int)a->bitems.size());
        for (int n = ns; n < nn; n++) {
            if (h->height[n] != L) continue;
            for (int fam = 0; fam < 2; fam++) {
                BItem b{};
                b.node = n;
                b.is_root = n == h->root;
                b.nchild = h->nson[n];
                b.ncls = ncls(n) == 4 ? 2 : 1;
                for (int k = 0; k < 2; k++) {
                    b.cls[k] = fam + 2 * k;
                    b.pslot[k] = k < b.ncls ? h->slot_of[n * 4 + b.cls[k]] : -1;
                    b.sslot[k] = (k < b.ncls && h->scale[n]) ? h->sslot_of[n * 4 + b.cls[k]] : -1;
                }
                for (int i = 0; i < MAXC; i++)
                    for (int k = 0; k < 2; k++) { b.pidx[i][k] = -1; b.tslot[i][k] = -1; }
                for (int i = 0; i < MAXC; i++) b.child[i] = i < b.nchild ? h->sons[n * MAXC + i] : -1;
                for (int i = 0; i < b.nchild; i++) {
                    int s = h->sons[n * MAXC + i];
                    for (int k = 0; k < b.ncls; k++) {
                        int c = b.cls[k];
                        int w = h->label[s] == 0 ? (c & 1) : (c <= 1 ? c : 2);
                        b.pidx[i][k] = h->pair_of[s * 3 + w];
                        b.tslot[i][k] = s < ns ? -1 : h->slot_of[s * 4 + cls_of(s, c)];
                    }
                    if (b.ncls == 1) { b.pidx[i][1] = b.pidx[i][0]; b.tslot[i][1] = b.tslot[i][0]; }
                }
                for (int k = 0; k < 2; k++) b.eslot[k] = b.pslot[k] >= 0 ? b.pslot[k] * MAXC : -1;
                a->bitems.push_back(b);
            }
        }
    }
    a->blevel_off.push_back((int)a->bitems.size());
    // checkpointed adjoint: E / Ebar rows numbered within each tree level
    // (slot -> its index among the items of its level)
    a->ckpt = h->precision == GB_PREC_FP64 && h->tune.checkpoint > 0;
    std::vector<int> erow((size_t)h->nslot, -1);
    for (int L = 0; L + 1 < (int)h->level_off.size(); L++)
        for (int q = h->level_off[L]; q < h->level_off[L + 1]; q++) erow[h->items[q].slot] = q - h->level_off[L];
    auto ebase = [&](int slot) { return a->ckpt ? erow[slot] * MAXC : slot * MAXC; };
    if (a->ckpt) {
        for (BItem &b : a->bitems)
            for (int k = 0; k < 2; k++) b.eslot[k] = b.pslot[k] >= 0 ? ebase(b.pslot[k]) : -1;
        a->ckpt_rows = 0;
        a->ritems.clear();
        a->rlevel_off.clear();
        a->plist.clear();
        a->plevel_off.clear();
        std::vector<char> seen(h->pairs.size(), 0);
        for (int L = (int)h->level_off.size() - 2; L >= 0; L--) {      // top-down, as the sweep
            a->rlevel_off.push_back((int)a->ritems.size());
            a->plevel_off.push_back((int)a->plist.size());
            a->ckpt_rows = std::max(a->ckpt_rows, h->level_off[L + 1] - h->level_off[L]);
            for (int q = h->level_off[L]; q < h->level_off[L + 1]; q++) {
                Item it = h->items[q];
                it.eslot = ebase(it.slot);
                a->ritems.push_back(it);
                for (int i = 0; i < it.nchild; i++)
                    if (!seen[it.pidx[i]]) {
                        seen[it.pidx[i]] = 1;
                        a->plist.push_back(it.pidx[i]);
                    }
            }
        }
        a->rlevel_off.push_back((int)a->ritems.size());
        a->plevel_off.push_back((int)a->plist.size());
    }
    // dlnL/dP contributions per pair
    std::vector<std::vector<Contrib>> per((size_t)h->pairs.size());
    for (const Item &it : h->items)
        for (int i = 0; i < it.nchild; i++) {
            Contrib cb{ebase(it.slot) + i, it.cslot[i], it.child[i]};
            per[it.pidx[i]].push_back(cb);
        }
    a->coff.assign(h->pairs.size() + 1, 0);
    for (size_t p = 0; p < per.size(); p++) {
        a->coff[p + 1] = a->coff[p] + (int)per[p].size();
        for (auto &c : per[p]) a->contrib.push_back(c);
    }
    // the FP64 kernel works in chunks of GCHUNK; the split-precision ones as
    // tuned, else GCHUNK_FAST halved (down to GCHUNK) until the (pair, chunk)
    // tasks are at least four per SM
    if (h->precision == GB_PREC_FP64) {
        a->gchunk = GCHUNK;
    } else if (h->tune.gchunk > 0) {
        a->gchunk = h->tune.gchunk;
    } else {
        int dev = 0, nsm = 152;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev))
            nsm = 152;
        a->gchunk = GCHUNK_FAST;
        while (a->gchunk > GCHUNK && (long)h->pairs.size() * ((h->npatt + a->gchunk - 1) / a->gchunk) < 4L * nsm)
            a->gchunk /= 2;
    }
    a->nchunk = (h->npatt + a->gchunk - 1) / a->gchunk;
    a->nfreq_blocks = (h->npatt + 255) / 256;
    const size_t npad = h->npad;
    int rc;
    if ((rc = dalloc(&a->d_bitems, a->bitems.size())) || (rc = dalloc(&a->d_contrib, a->contrib.size())) ||
        (rc = dalloc(&a->d_coff, a->coff.size())) ||
        (rc = dalloc(&a->d_Ebar, (size_t)(a->ckpt ? a->ckpt_rows : h->nslot) * MAXC * npad * 64)) ||
        (a->ckpt && !h->d_E && (rc = dalloc(&h->d_E, (size_t)a->ckpt_rows * MAXC * npad * 64))) ||
        (a->ckpt && (rc = dalloc(&a->d_ritems, a->ritems.size()))) ||
        (a->ckpt && (rc = dalloc(&a->d_plist, std::max<size_t>(a->plist.size(), 1)))) ||
        (rc = dalloc(&a->d_Abar, (size_t)h->nslot * npad * 64)) ||
        (rc = dalloc(&a->d_Gpart, h->pairs.size() * a->nchunk * 64 * 64)) ||
        (rc = dalloc(&a->d_Dm, DM_MATS * 64 * 64)) ||
        (h->precision != GB_PREC_FP64 && (rc = dalloc(&a->d_UVdf, UVDF_DM + DM_MATS * 64 * 64))) || (rc = dalloc(&a->d_pout, h->pairs.size() * 3)) ||
        (rc = dalloc(&a->d_fpart, a->nfreq_blocks * 4)) || (rc = dalloc(&a->d_gp, 1)))
        return rc;
    if (cudaMallocHost((void **)&a->h_gp, sizeof(GradParams)) ||
        cudaMallocHost((void **)&a->h_pout, sizeof(double) * h->pairs.size() * 3) ||
        cudaMallocHost((void **)&a->h_fpart, sizeof(double) * a->nfreq_blocks * 4))
        return fail(GB_ERR_OOM, "cudaMallocHost (adjoint)");
    CK(cudaMemcpy(a->d_bitems, a->bitems.data(), sizeof(BItem) * a->bitems.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(a->d_contrib, a->contrib.data(), sizeof(Contrib) * std::max<size_t>(a->contrib.size(), 1), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(a->d_coff, a->coff.data(), sizeof(int) * a->coff.size(), cudaMemcpyHostToDevice));
    if (a->ckpt) {
        CK(cudaMemcpy(a->d_ritems, a->ritems.data(), sizeof(Item) * a->ritems.size(), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(a->d_plist, a->plist.data(), sizeof(int) * a->plist.size(), cudaMemcpyHostToDevice));
    }
    // the Ebar rows of padded patterns must be zero for the dP reduction: they are
    // written by the sweep with g = 0 (fpatt = 0) at the root and products below
    CK(cudaMemset(a->d_Abar, 0, sizeof(double) * (size_t)h->nslot * npad * 64));
    CK(cudaFuncSetAttribute(gradP_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGradPSmem));
    CK(cudaFuncSetAttribute(gradH_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGradHSmem));
    CK(cudaFuncSetAttribute(gradH_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGradHdfSmem));
    CK(cudaFuncSetAttribute(gradH_batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGradHdfSmem));
    return 0;
}

void launch_dmat(gb_handle *h) {
    dmat_kernel<<<DM_BLOCKS, 256, 0, h->stream>>>(h->d_prm, h->adj->d_gp, h->adj->d_Dm, h->adj->d_UVdf);
}

void launch_gradH(gb_handle *h) {
    AdjointState *a = h->adj;
    gradH_kernel<<<(unsigned)h->pairs.size(), 256, kGradHSmem, h->stream>>>(h->d_pairs, h->d_label, h->d_tnode,
                                                                           h->d_prm, a->d_Gpart, a->nchunk,
                                                                           a->d_Dm, a->d_pout);
}

void launch_gradH_df(gb_handle *h) {
    AdjointState *a = h->adj;
    gradH_df_kernel<<<(unsigned)h->pairs.size(), 256, kGradHdfSmem, h->stream>>>(
        h->d_pairs, h->d_label, h->d_tnode, h->d_prm, reinterpret_cast<const float2 *>(a->d_Gpart), a->nchunk,
        a->d_Dm, a->d_UVdf, a->d_pout);
}

void launch_dmat_batched(const DmatArgs *args, const int2 *map, int nblocks, cudaStream_t st) {
    if (nblocks > 0) dmat_batched_kernel<<<nblocks, 256, 0, st>>>(args, map);
}

void launch_gradH_batched(const GradHArgs *args, const int2 *map, int nblocks, cudaStream_t st) {
    if (nblocks > 0) gradH_batched_kernel<<<nblocks, 256, kGradHdfSmem, st>>>(args, map);
}

void launch_freq_batched(const FreqArgs *args, const int2 *map, int nblocks, cudaStream_t st) {
    if (nblocks > 0) freq_batched_kernel<<<nblocks, 256, 0, st>>>(args, map);
}

// the FP64 gradient kernels on explicit buffers (clade models, clade.cu)
cudaError_t init_fp64_adjoint_kernels() {
    cudaError_t e = cudaFuncSetAttribute(gradP_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGradPSmem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(gradH_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kGradHSmem);
}

void launch_dmat_fp64(const DevParams *prm, const GradParams *gp, double *Dm, cudaStream_t st) {
    dmat_kernel<<<DM_BLOCKS, 256, 0, st>>>(prm, gp, Dm, nullptr);
}

void launch_bwd_level_fp64(const BItem *bitems, int nitems, int ntile, int npad, const double *Pt, const double *E,
                           double *Ebar, double *Abar, const double *scaleF, const double *fpatt, const double *post,
                           const double *fbar, const double *pi, cudaStream_t st) {
    dim3 grid(ntile, nitems);
    bwd_level_kernel<<<grid, 128, 0, st>>>(bitems, npad, Pt, E, Ebar, Abar, scaleF, fpatt, post, fbar, pi);
}

void launch_gradP_fp64(const Contrib *contrib, const int *coff, int npair, int nchunk, int npatt, int npad,
                       const double *Ebar, const double *conP, const unsigned char *z, double *Gpart,
                       const unsigned char *amb, cudaStream_t st) {
    dim3 grid((unsigned)npair, nchunk);
    gradP_kernel<<<grid, 128, kGradPSmem, st>>>(contrib, coff, npatt, npad, Ebar, conP, z, Gpart, nchunk, amb,
                                                nullptr);
}

void launch_gradH_fp64(const PairDesc *pairs, int npair, const int *label, const double *tnode, const DevParams *prm,
                       const double *Gpart, int nchunk, const double *Dm, double *pout, cudaStream_t st) {
    if (npair > 0)
        gradH_kernel<<<(unsigned)npair, 256, kGradHSmem, st>>>(pairs, label, tnode, prm, Gpart, nchunk, Dm, pout);
}

void launch_freq_fp64(const double *fhK, const double *lnf, const double *fpatt, int npatt, int npad, int nscale,
                      double *fpart, cudaStream_t st) {
    freq_kernel<<<(npatt + 255) / 256, 256, 0, st>>>(fhK, lnf, fpatt, npatt, npad, nscale, fpart);
}

void launch_freq(gb_handle *h, int nscale) {
    AdjointState *a = h->adj;
    freq_kernel<<<a->nfreq_blocks, 256, 0, h->stream>>>(h->d_fhK, h->d_lnf, h->d_fpatt, h->npatt, h->npad,
                                                       nscale, a->d_fpart);
}

namespace {

int record_backward(gb_handle *h) {
    AdjointState *a = h->adj;
    int nk = 0;
    dmat_kernel<<<DM_BLOCKS, 256, 0, h->stream>>>(h->d_prm, a->d_gp, a->d_Dm, nullptr);
    prof_mark(h, GB_K_OTHER);
    nk++;
    for (size_t L = 0; L + 1 < a->blevel_off.size(); L++) {
        int n = a->blevel_off[L + 1] - a->blevel_off[L];
        if (!n) continue;
        if (a->ckpt) {
            // this level's edge messages again (the forward kept none): the
            // level's items with level-local E rows; conditional likelihoods,
            // scale factors and root sums are rewritten with the same values
            const int nr = a->rlevel_off[L + 1] - a->rlevel_off[L];
            launch_prune_fp64(a->d_ritems + a->rlevel_off[L], nr, h->ntile, h->npad, h->d_z, h->d_Pt, h->d_conP,
                              h->d_E, h->d_scaleF, h->d_scale_list, h->nscale, h->d_pi, h->d_fbar, h->d_ssum,
                              h->d_fhK, h->stream, h->d_amb);
            prof_mark(h, GB_K_PRUNE);
            nk++;
        }
        dim3 grid(h->ntile, n);
        bwd_level_kernel<<<grid, 128, 0, h->stream>>>(a->d_bitems + a->blevel_off[L], h->npad, h->d_Pt,
                                                      h->d_E, a->d_Ebar, a->d_Abar, h->d_scaleF,
                                                      h->d_fpatt, h->d_post, h->d_fbar, h->d_pi);
        prof_mark(h, GB_K_BWD);
        nk++;
        if (a->ckpt) {      // the level's pairs, while its Ebar rows are there
            const int np = a->plevel_off[L + 1] - a->plevel_off[L];
            if (np) {
                dim3 g2((unsigned)np, a->nchunk);
                gradP_kernel<<<g2, 128, kGradPSmem, h->stream>>>(a->d_contrib, a->d_coff, h->npatt, h->npad,
                                                                 a->d_Ebar, h->d_conP, h->d_z, a->d_Gpart,
                                                                 a->nchunk, h->d_amb, a->d_plist + a->plevel_off[L]);
                prof_mark(h, GB_K_GRADP);
                nk++;
            }
        }
    }
    if (!a->ckpt) {
        dim3 g2((unsigned)h->pairs.size(), a->nchunk);
        gradP_kernel<<<g2, 128, kGradPSmem, h->stream>>>(a->d_contrib, a->d_coff, h->npatt, h->npad, a->d_Ebar,
                                                         h->d_conP, h->d_z, a->d_Gpart, a->nchunk, h->d_amb,
                                                         nullptr);
        prof_mark(h, GB_K_GRADP);
        nk++;
    }
    gradH_kernel<<<(unsigned)h->pairs.size(), 256, kGradHSmem, h->stream>>>(h->d_pairs, h->d_label, h->d_tnode,
                                                                   h->d_prm, a->d_Gpart, a->nchunk,
                                                                   a->d_Dm, a->d_pout);
    prof_mark(h, GB_K_GRADH);
    nk++;
    freq_kernel<<<a->nfreq_blocks, 256, 0, h->stream>>>(h->d_fhK, h->d_lnf, h->d_fpatt, h->npatt,
                                                       h->npad, h->nscale, a->d_fpart);
    prof_mark(h, GB_K_OTHER);
    nk++;
    return nk;
}

}  // namespace

int adjoint_record(gb_handle *h) { return record_backward(h); }

bool adjoint_ready(gb_handle *h) { return h->adj && h->adj->graph; }

int adjoint_launch_graph(gb_handle *h) {
    CK(cudaGraphLaunch(h->adj->graph, h->stream));
    return 0;
}

int adjoint_run(gb_handle *h, const Derived *D, const ModelParams &m, const double *blength,
                gb_grad *grad, gb_stats *stats) {
    if (!h->adj) {
        int rc = adjoint_init(h);
        if (rc) return rc;
    }
    AdjointState *a = h->adj;
    if (!a->graph) {
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        a->graph_kernels = record_backward(h);
        CK(cudaStreamEndCapture(h->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&a->graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate (adjoint)");
    }
    std::memcpy(a->h_gp->dQk, D->dQk, sizeof(D->dQk));
    std::memcpy(a->h_gp->dQw, D->dQw, sizeof(D->dQw));
    CK(cudaEventRecord(h->ev0, h->stream));
    CK(cudaMemcpyAsync(a->d_gp, a->h_gp, sizeof(GradParams), cudaMemcpyHostToDevice, h->stream));
    CK(cudaGraphLaunch(a->graph, h->stream));
    const size_t np = h->pairs.size();
    int rcf = adjoint_fetch(h);
    if (rcf) return rcf;
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaGetLastError());
    h->kernels_last += a->graph_kernels;
    if (stats) {
        float ms = 0;
        cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        stats->ms_device += ms;
        stats->kernels += a->graph_kernels;
        stats->h2d_bytes += sizeof(GradParams);
        stats->d2h_bytes += sizeof(double) * (np * 3 + a->nfreq_blocks * 4);
    }

    adjoint_chain(h, D, blength, grad);
    (void)m;
    return 0;
}

int adjoint_fetch(gb_handle *h) {
    AdjointState *a = h->adj;
    const size_t np = h->pairs.size();
    CK(cudaMemcpyAsync(a->h_pout, a->d_pout, sizeof(double) * np * 3, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(a->h_fpart, a->d_fpart, sizeof(double) * a->nfreq_blocks * 4, cudaMemcpyDeviceToHost, h->stream));
    return 0;
}

void adjoint_chain(gb_handle *h, const Derived *D, const double *blength, gb_grad *grad) {
    AdjointState *a = h->adj;
    const size_t np = h->pairs.size();
    // chain rule on the host (all derivatives of lnL; negated at the end)
    const int nn = h->nnode;
    std::vector<double> dtp(nn, 0.0);    // dlnL/dt' per node
    double dk = 0, dw0 = 0, dw1 = 0, dw2 = 0;
    for (size_t p = 0; p < np; p++) {
        const PairDesc &pd = h->pairs[p];
        dtp[pd.node] += a->h_pout[p * 3 + 0];
        dk += a->h_pout[p * 3 + 1];
        if (pd.w == 0) dw0 += a->h_pout[p * 3 + 2];
        if (pd.w == 1) dw1 += a->h_pout[p * 3 + 2];     // model B's w1 (zero under model A)
        if (pd.w == 2) dw2 += a->h_pout[p * 3 + 2];
    }
    double dqf[2] = {0, 0};
    for (int n = 0; n < nn; n++) {
        if (n == h->root) continue;
        const int b = h->label[n];
        const double t = blength[n];
        grad->d_blength[n] = -(dtp[n] * D->qf[b]);
        dqf[b] += dtp[n] * t;
    }
    grad->d_blength[h->root] = 0.0;
    double dfk[4] = {0, 0, 0, 0};   // sum_h fpatt f_c / R
    for (int b = 0; b < a->nfreq_blocks; b++)
        for (int c = 0; c < 4; c++) dfk[c] += a->h_fpart[b * 4 + c];
    double gk = dk, gw0 = dw0, gw1 = dw1, gw2 = dw2, gp0 = 0, gp1 = 0;
    for (int b = 0; b < 2; b++) {
        gk += dqf[b] * D->dqf[b][0];
        gw0 += dqf[b] * D->dqf[b][1];
        gw2 += dqf[b] * D->dqf[b][2];
        gp0 += dqf[b] * D->dqf[b][3];
        gp1 += dqf[b] * D->dqf[b][4];
        gw1 += dqf[b] * D->dqf[b][5];
    }
    a->d_omega1 = -gw1;
    for (int c = 0; c < 4; c++) {
        gp0 += dfk[c] * D->dfreqK[c][0];
        gp1 += dfk[c] * D->dfreqK[c][1];
    }
    grad->d_kappa = -gk;
    grad->d_omega0 = -gw0;
    grad->d_omega2 = -gw2;
    grad->d_p0 = -gp0;
    grad->d_p1 = -gp1;
}

}  // namespace gb
