// FP64 kernels of the drop-in path.
//
//   pmat_fp64   P(t) = U diag(exp(Root t)) V for every unique (branch, omega)
//               pair, stored transposed and zero padded to 64x64.  With the
//               codon frequencies given, U and V come from the symmetrised
//               eigenproblem (V[m][k] = U[k][m] pi_k, eigen_qrev), so
//               P[j][k] = pi_k S[j][k] with S = U diag(e) U^T symmetric: only
//               its upper-triangular 8 x 8 blocks are formed (36 of 64).
//               (PMatUVRoot tools.c:515-546: negatives clamped to 0, t < 1e-100
//               gives the identity; cuda-codeml.cu:679-742 computes the same per
//               node and class, here once per unique pair).
//   prune_fp64  one CTA per (32-pattern tile, node, class) slot of a tree level:
//               the products of all children's messages (tip gathers and
//               (32x61)x(61x61) FP64 contractions) are fused into the parent's
//               tile, followed by codeml's per-pattern node scaling and, at the
//               root, the pi-weighted sum and log (ConditionalPNode
//               codeml.c:3402-3459, NodeScale treesub.c:6940-6975, fx_r
//               treesub.c:7512-7538).
//   mix         the site-class mixture, per-pattern log f and the fpatt-weighted
//               sum with a deterministic two-level reduction (lfundG
//               treesub.c:7342-7394).
#include <cuda_runtime.h>

#include "internal.h"
#include "batch_internal.h"

namespace gb {

namespace {

constexpr int NC = 61;

__device__ __forceinline__ void pmat_body(const PairDesc *__restrict__ pairs, const int *__restrict__ label,
                                          const double *__restrict__ tnode, const DevParams *__restrict__ prm,
                                          double *__restrict__ Pt, int pair, const double *__restrict__ pi) {
    extern __shared__ double sm[];
    double *UeT = sm;             // [61][64]: UeT[m][j] = U[j][m] e^{Root_m t}
    double *Vs = sm + NC * 64;    // [61][64]: Vs[m][k] = V[m][k] (symmetric form: U[k][m])
    const PairDesc pd = pairs[pair];
    const int w = pd.w;
    const double t = tnode[pd.node] * prm->qf[label[pd.node]];
    double *out = Pt + (size_t)pair * 64 * 64;
    const int tid = threadIdx.x;
    if (t < 1e-100) {
        for (int i = tid; i < 64 * 64; i += blockDim.x) out[i] = (i / 64 == i % 64 && i / 64 < NC) ? 1.0 : 0.0;
        return;
    }
    const double *U = prm->U[w];
    const double *V = prm->V[w];
    if (pi && !prm->sym) pi = nullptr;                // general U, V: the full product (the flag is read only
                                                      // with pi: callers without it pass a shorter model block)
    __shared__ double ex[64];
    if (tid < NC) ex[tid] = exp(t * prm->Root[w][tid]);
    __syncthreads();
    for (int i = tid; i < NC * 64; i += blockDim.x) {
        int m = i / 64, c = i % 64;
        UeT[i] = c < NC ? U[c * NC + m] * ex[m] : 0.0;
        Vs[i] = c < NC ? (pi ? U[c * NC + m] : V[m * NC + c]) : 0.0;
    }
    __syncthreads();
    if (pi) {
        // S[j][k] on the 36 upper-triangular 8 x 8 blocks (R <= C): thread tid
        // takes entry (tid mod 64) of blocks 4q + tid / 64, q = 0..8; then
        // Pt[k][j] = P[j][k] = pi_k S[j][k] and Pt[j][k] = pi_j S[j][k]
        const int e = tid & 63, i8 = e >> 3, j8 = e & 7;
#pragma unroll 1
        for (int q = 0; q < 9; q++) {
            int u = 4 * q + (tid >> 6), R = 0;
            while (u >= 8 - R) {                      // block u of rows R, R+1, ... (8 - R blocks in row R)
                u -= 8 - R;
                R++;
            }
            const int C = R + u;
            if (R == C && i8 > j8) continue;          // a diagonal block's lower half is the upper one mirrored
            const int j = 8 * R + i8, k = 8 * C + j8;
            double acc = 0.0;
            for (int m = 0; m < NC; m++) acc = fma(UeT[m * 64 + j], Vs[m * 64 + k], acc);
            const bool in = j < NC && k < NC;
            double pjk = in ? acc * pi[k] : 0.0, pkj = in ? acc * pi[j] : 0.0;
            if (pjk < 0.0) pjk = 0.0;
            if (pkj < 0.0) pkj = 0.0;
            out[k * 64 + j] = pjk;
            out[j * 64 + k] = pkj;
        }
        return;
    }
    // thread -> row k of Pt (child state), 16 consecutive parent states j
    const int k = tid >> 2;
    const int j0 = (tid & 3) * 16;
    double acc[16];
#pragma unroll
    for (int i = 0; i < 16; i++) acc[i] = 0.0;
    for (int m = 0; m < NC; m++) {
        const double v = Vs[m * 64 + k];
        const double *ue = UeT + m * 64 + j0;
#pragma unroll
        for (int i = 0; i < 16; i++) acc[i] = fma(ue[i], v, acc[i]);
    }
#pragma unroll
    for (int i = 0; i < 16; i++) {
        double p = acc[i];
        if (p < 0.0 || k >= NC) p = 0.0;
        out[k * 64 + j0 + i] = p;
    }
}

__global__ void __launch_bounds__(256) pmat_fp64_kernel(const PairDesc *__restrict__ pairs,
                                                        const int *__restrict__ label,
                                                        const double *__restrict__ tnode,
                                                        const DevParams *__restrict__ prm,
                                                        double *__restrict__ Pt,
                                                        const double *__restrict__ pi) {
    pmat_body(pairs, label, tnode, prm, Pt, blockIdx.x, pi);
}

// many genes in one launch: block b works on pair map[b].y of gene map[b].x
__global__ void __launch_bounds__(256) pmat_batched_kernel(const PmatArgs *__restrict__ args,
                                                           const int2 *__restrict__ map) {
    const int2 g = map[blockIdx.x];
    const PmatArgs &a = args[g.x];
    pmat_body(a.pairs, a.label, a.tnode, a.prm, a.Pt, g.y, a.pi);
}

// 128 threads: row group rg = tid/16 owns tile rows 4rg..4rg+3, column group
// cg = tid%16 owns states 4cg..4cg+3.
__global__ void __launch_bounds__(128) prune_fp64_kernel(
    const Item *__restrict__ items, int npad, const unsigned char *__restrict__ z,
    const double *__restrict__ Pt, double *__restrict__ conP, double *__restrict__ E,
    double *__restrict__ scaleF, const int *__restrict__ scale_list, int nscale,
    const double *__restrict__ pi, double *__restrict__ fbar, double *__restrict__ ssum,
    double *__restrict__ fhK, const unsigned char *__restrict__ amb) {
    __shared__ double Ps[NC * 64];          // rows k < 61 of Pt
    __shared__ double Ls[TILE64 * 65];
    const Item it = items[blockIdx.y];
    const int tile = blockIdx.x;
    const int h0 = tile * TILE64;
    const int tid = threadIdx.x;
    const int rg = tid >> 4, cg = tid & 15;
    const int r0 = rg * 4, c0 = cg * 4;

    double acc[4][4];
    for (int ci = 0; ci < it.nchild; ci++) {
        const double *P = Pt + (size_t)it.pidx[ci] * 64 * 64;
        __syncthreads();
        for (int i = tid; i < NC * 64 / 2; i += 128)
            reinterpret_cast<double2 *>(Ps)[i] = reinterpret_cast<const double2 *>(P)[i];
        double tmp[4][4];
        if (it.cslot[ci] < 0) {
            __syncthreads();
            const unsigned char *zc = z + (size_t)it.child[ci] * npad + h0 + r0;
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int zz = zc[r];
                if (zz < NC || !amb) {
#pragma unroll
                    for (int c = 0; c < 4; c++) tmp[r][c] = Ps[zz * 64 + c0 + c];
                } else {
                    // an ambiguous codon: the sum over the sense codons it stands
                    // for, in codeml's CharaMap order (codeml.c:3438-3445)
                    const unsigned char *map = amb + 256 + 64 * zz;
#pragma unroll
                    for (int c = 0; c < 4; c++) tmp[r][c] = 0.0;
                    for (int q = 0; q < amb[zz]; q++)
#pragma unroll
                        for (int c = 0; c < 4; c++) tmp[r][c] += Ps[map[q] * 64 + c0 + c];
                }
            }
        } else {
            const double *L = conP + ((size_t)it.cslot[ci] * npad + h0) * 64;
            for (int i = tid; i < TILE64 * 64; i += 128) Ls[(i >> 6) * 65 + (i & 63)] = L[i];
            __syncthreads();
#pragma unroll
            for (int r = 0; r < 4; r++)
#pragma unroll
                for (int c = 0; c < 4; c++) tmp[r][c] = 0.0;
#pragma unroll 4
            for (int k = 0; k < NC; k++) {
                double a[4], b[4];
#pragma unroll
                for (int r = 0; r < 4; r++) a[r] = Ls[(r0 + r) * 65 + k];
#pragma unroll
                for (int c = 0; c < 4; c++) b[c] = Ps[k * 64 + c0 + c];
#pragma unroll
                for (int r = 0; r < 4; r++)
#pragma unroll
                    for (int c = 0; c < 4; c++) tmp[r][c] = fma(a[r], b[c], tmp[r][c]);
            }
        }
        if (E) {
            double *e = E + ((size_t)(it.eslot + ci) * npad + h0 + r0) * 64 + c0;
#pragma unroll
            for (int r = 0; r < 4; r++)
                *reinterpret_cast<double4 *>(e + r * 64) = make_double4(tmp[r][0], tmp[r][1], tmp[r][2], tmp[r][3]);
        }
#pragma unroll
        for (int r = 0; r < 4; r++)
#pragma unroll
            for (int c = 0; c < 4; c++) acc[r][c] = ci == 0 ? tmp[r][c] : acc[r][c] * tmp[r][c];
    }

    if (it.sslot >= 0) {
#pragma unroll
        for (int r = 0; r < 4; r++) {
            double m = 0.0;
#pragma unroll
            for (int c = 0; c < 4; c++)
                if (c0 + c < NC && acc[r][c] > m) m = acc[r][c];
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
            double sf;
            if (m < 1e-300) {
#pragma unroll
                for (int c = 0; c < 4; c++) acc[r][c] = (c0 + c < NC) ? 1.0 : 0.0;
                sf = -800.0;
            } else {
#pragma unroll
                for (int c = 0; c < 4; c++) acc[r][c] = acc[r][c] / m;
                sf = log(m);
            }
            if (cg == 0) scaleF[(size_t)it.sslot * npad + h0 + r0 + r] = sf;
        }
    }

    if (!it.is_root) {
        double *o = conP + ((size_t)it.slot * npad + h0 + r0) * 64 + c0;
#pragma unroll
        for (int r = 0; r < 4; r++)
            *reinterpret_cast<double4 *>(o + r * 64) = make_double4(acc[r][0], acc[r][1], acc[r][2], acc[r][3]);
        return;
    }
    // root: f~_h = sum_i pi_i L_root[h][i]; codeml's fhK = log f + sum of scale logs
    double pic[4];
#pragma unroll
    for (int c = 0; c < 4; c++) pic[c] = (c0 + c < NC) ? pi[c0 + c] : 0.0;
#pragma unroll
    for (int r = 0; r < 4; r++) {
        double f = 0.0;
#pragma unroll
        for (int c = 0; c < 4; c++) f = fma(pic[c], acc[r][c], f);
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
        if (cg == 0) {
            const int h = h0 + r0 + r;
            if (f <= 0.0) f = 1e-300;
            // scale logs in node order, added to log f one by one as fx_r does
            double s = 0.0, v = nscale > 0 ? log(f) : f;
            for (int k = 0; k < nscale; k++) {
                const double sf = scaleF[(size_t)scale_list[it.cls * nscale + k] * npad + h];
                s += sf;
                v += sf;
            }
            fbar[(size_t)it.cls * npad + h] = f;
            ssum[(size_t)it.cls * npad + h] = s;
            fhK[(size_t)it.cls * npad + h] = v;
        }
    }
}

// mixture over the 4 classes, log, fpatt-weighted sum; post[c][h] = class posterior
__device__ __forceinline__ void mix_body(const double *__restrict__ fhK, const double *__restrict__ fpatt,
                                         const DevParams *__restrict__ prm, int npatt, int npad, int nscale,
                                         double *__restrict__ lnf, double *__restrict__ post,
                                         double *__restrict__ partial, unsigned *__restrict__ ticket,
                                         double *__restrict__ out, int bid, int nb,
                                         const double *__restrict__ fbar, float2 *__restrict__ groot) {
    __shared__ double red[256];
    __shared__ bool last;
    const int h = bid * blockDim.x + threadIdx.x;
    double contrib = 0.0;
    if (h < npatt) {
        double v[4], fk[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            v[c] = fhK[(size_t)c * npad + h];
            fk[c] = prm->freqK[c];
        }
        double fh, q[4];
        if (nscale > 0) {
            int itop = 0;
#pragma unroll
            for (int c = 1; c < 4; c++)
                if (v[c] > v[itop]) itop = c;
            const double t = v[itop];
            double s = 0.0;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                q[c] = fk[c] * exp(v[c] - t);
                s += q[c];
            }
            fh = t + log(s);
#pragma unroll
            for (int c = 0; c < 4; c++) q[c] /= s;
        } else {
            double s = 0.0;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                q[c] = fk[c] * v[c];
                s += q[c];
            }
            const double sp = s <= 0.0 ? 1e-300 : s;
#pragma unroll
            for (int c = 0; c < 4; c++) q[c] /= sp;
            fh = log(sp);
        }
        const double fp = fpatt[h];
        if (fp > 0.0) contrib = fh * fp;
        if (lnf) lnf[h] = fp > 0.0 ? fh : 0.0;
        if (post)
#pragma unroll
            for (int c = 0; c < 4; c++) post[(size_t)c * npad + h] = q[c];
        if (groot)      // dlnL/df~_c = fpatt post_c / f~_c, the adjoint's root seed
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const double f = fbar[(size_t)c * npad + h];
                const double g = (fp > 0.0 && f > 0.0) ? fp * q[c] / f : 0.0;
                const float gh = (float)g;
                groot[(size_t)c * npad + h] = make_float2(gh, (float)(g - (double)gh));
            }
    }
    red[threadIdx.x] = contrib;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[bid] = red[0];
        __threadfence();
        unsigned prev = atomicAdd(ticket, 1u);
        last = (prev == (unsigned)nb - 1);
    }
    __syncthreads();
    if (last) {
        // the last block sums the block partials in a fixed order
        __threadfence();
        double s = 0.0;
        for (int i = threadIdx.x; i < nb; i += blockDim.x) s += ((volatile double *)partial)[i];
        red[threadIdx.x] = s;
        __syncthreads();
        for (int k = 128; k > 0; k >>= 1) {
            if (threadIdx.x < k) red[threadIdx.x] += red[threadIdx.x + k];
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            out[0] = -red[0];
            *ticket = 0u;
        }
    }
}

__global__ void __launch_bounds__(256) mix_kernel(const double *__restrict__ fhK,
                                                  const double *__restrict__ fpatt,
                                                  const DevParams *__restrict__ prm, int npatt,
                                                  int npad, int nscale, double *__restrict__ lnf,
                                                  double *__restrict__ post,
                                                  double *__restrict__ partial,
                                                  unsigned *__restrict__ ticket,
                                                  double *__restrict__ out,
                                                  const double *__restrict__ fbar,
                                                  float2 *__restrict__ groot) {
    mix_body(fhK, fpatt, prm, npatt, npad, nscale, lnf, post, partial, ticket, out, blockIdx.x, gridDim.x,
             fbar, groot);
}

__global__ void __launch_bounds__(256) mix_batched_kernel(const MixArgs *__restrict__ args,
                                                          const int2 *__restrict__ map) {
    const int2 g = map[blockIdx.x];
    const MixArgs &a = args[g.x];
    mix_body(a.fhK, a.fpatt, a.prm, a.npatt, a.npad, a.nscale, a.lnf, a.post, a.partial, a.ticket, a.out, g.y,
             a.nblocks, a.fbar, a.groot);
}

}  // namespace

constexpr int kPmatSmem = 2 * NC * 64 * sizeof(double);

cudaError_t init_fp64_kernels() {
    cudaError_t e = cudaFuncSetAttribute(pmat_fp64_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPmatSmem);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(pmat_batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kPmatSmem);
}

void launch_pmat_batched(const PmatArgs *args, const int2 *map, int nblocks, cudaStream_t st) {
    if (nblocks > 0) pmat_batched_kernel<<<nblocks, 256, kPmatSmem, st>>>(args, map);
}

void launch_mix_batched(const MixArgs *args, const int2 *map, int nblocks, cudaStream_t st) {
    if (nblocks > 0) mix_batched_kernel<<<nblocks, 256, 0, st>>>(args, map);
}

void launch_pmat_fp64(const PairDesc *pairs, int npair, const int *label, const double *tnode,
                      const DevParams *prm, double *Pt, cudaStream_t st, const double *pi) {
    pmat_fp64_kernel<<<npair, 256, kPmatSmem, st>>>(pairs, label, tnode, prm, Pt, pi);
}

void launch_prune_fp64(const Item *items, int nitems, int ntile, int npad, const unsigned char *z,
                       const double *Pt, double *conP, double *E, double *scaleF,
                       const int *scale_list, int nscale, const double *pi, double *fbar,
                       double *ssum, double *fhK, cudaStream_t st, const unsigned char *amb) {
    dim3 grid(ntile, nitems);
    prune_fp64_kernel<<<grid, 128, 0, st>>>(items, npad, z, Pt, conP, E, scaleF, scale_list,
                                            nscale, pi, fbar, ssum, fhK, amb);
}

void launch_mix(const double *fhK, const double *fpatt, const DevParams *prm, int npatt, int npad,
                int nscale, double *lnf, double *post, double *partial, unsigned *ticket,
                double *out, cudaStream_t st, const double *fbar, float2 *groot) {
    int nb = (npatt + 255) / 256;
    mix_kernel<<<nb, 256, 0, st>>>(fhK, fpatt, prm, npatt, npad, nscale, lnf, post, partial, ticket, out, fbar,
                                   groot);
}

}  // namespace gb
