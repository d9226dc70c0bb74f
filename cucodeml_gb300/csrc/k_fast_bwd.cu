// Split-precision adjoint kernels (GB_PREC_FAST with a gradient).
//
// Same scheme as k_fast.cu, in normalised space: the forward stores each
// node's rows L~ (max in [0.5, 1)) and exponents, with
//   L~_a = 2^{-sh_a} prod_i E_i,   E_i = P_i L~_{s_i},   sh_a = expo_a - sum_i expo_{s_i},
// so that, holding the exact power-of-two shifts constant,
//   Ebar_i = A_a 2^{-sh_a} prod_{i' != i} E_i'          (double-float, SIMT)
//   A_{s_i} += Ebar_i P_i                                 (digit planes, tensor cores)
//   dlnL/dP_i += sum_h Ebar_i[h]^T L~_{s_i}[h]            (digit planes, tensor cores; tips: FP64 scatter)
// with A_root = fpatt rho / f~ * pi.  Ebar and A rows are renormalised like L~
// and carry their own exponents; all of them are non-negative and cut into
// balanced digits (|d| <= 128), so the tensor-core sums over 64 patterns stay
// within NS * 64 * 128^2 <= 2^23 and exact.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "adjoint_internal.h"
#include "fast_device.cuh"
#include "fast_internal.h"

namespace gb {

namespace {

using namespace fastdev;
constexpr int NC = 61;
constexpr int GSUB = 64;   // patterns per exact sub-chunk of dlnL/dP

__device__ __forceinline__ void load_row_block(const float2 *base, int t, float2 (&v)[8][4]) {
    // rows base (row0) and base + 8*64 (row0 + 8), columns 8nt + 2t, +1
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        const float4 a = *reinterpret_cast<const float4 *>(base + nt * 8 + 2 * t);
        const float4 b = *reinterpret_cast<const float4 *>(base + 8 * 64 + nt * 8 + 2 * t);
        v[nt][0] = make_float2(a.x, a.y); v[nt][1] = make_float2(a.z, a.w);
        v[nt][2] = make_float2(b.x, b.y); v[nt][3] = make_float2(b.z, b.w);
    }
}

__device__ __forceinline__ void store_row_block(float2 *base, int t, const float2 (&v)[8][4]) {
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
        *reinterpret_cast<float4 *>(base + nt * 8 + 2 * t) = make_float4(v[nt][0].x, v[nt][0].y, v[nt][1].x, v[nt][1].y);
        *reinterpret_cast<float4 *>(base + 8 * 64 + nt * 8 + 2 * t) = make_float4(v[nt][2].x, v[nt][2].y, v[nt][3].x, v[nt][3].y);
    }
}

// One CTA per (128-pattern tile, backward item).  Thread layout as in the
// forward: rows row0 = 16w + g and row0 + 8, columns 8nt + 2t, +1.
template <int NS>
__global__ void __launch_bounds__(256, 1) bwd_fast_kernel(FastBwdArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __nv_bfloat16 *As = reinterpret_cast<__nv_bfloat16 *>(smraw);
    __nv_bfloat16 *Bs = As + Smem<NS>::A_ELEMS;
    const BItem it = a.bitems[blockIdx.y];
    const int h0 = blockIdx.x * MT;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int row0 = warp * 16 + g;
    const size_t npad = a.npad;

    // exponent of A_a 2^{-sh_a} per class and row
    int eAs[2][2];
    for (int k = 0; k < it.ncls; k++) {
        const int c = it.cls[k];
#pragma unroll
        for (int r = 0; r < 2; r++) {
            const size_t h = h0 + row0 + 8 * r;
            const int ep = it.is_root ? a.expo_root[(size_t)c * npad + h] : a.expo[(size_t)it.pslot[k] * npad + h];
            int ec = 0;
            for (int i = 0; i < it.nchild; i++)
                if (it.tslot[i][k] >= 0) ec += a.expo[(size_t)it.tslot[i][k] * npad + h];
            eAs[k][r] = -(ep - ec);
        }
    }

    for (int i = 0; i < it.nchild; i++) {
        for (int k = 0; k < it.ncls; k++) {
            const int c = it.cls[k];
            float2 X[8][4];
            int eX[2];
            if (it.is_root) {
#pragma unroll
                for (int r = 0; r < 2; r++) {
                    const size_t h = h0 + row0 + 8 * r;
                    const double gsc = a.fpatt[h] * a.post[(size_t)c * npad + h] / a.fbar[(size_t)c * npad + h];
#pragma unroll
                    for (int nt = 0; nt < 8; nt++)
#pragma unroll
                        for (int q = 0; q < 2; q++) {
                            const int col = nt * 8 + 2 * t + q;
                            const double v = col < NC ? gsc * a.pi[col] : 0.0;
                            const float hi = (float)v;
                            X[nt][2 * r + q] = make_float2(hi, (float)(v - (double)hi));
                        }
                    eX[r] = eAs[k][r];
                }
            } else {
                load_row_block(a.Abar + ((size_t)it.pslot[k] * npad + h0 + row0) * 64, t, X);
#pragma unroll
                for (int r = 0; r < 2; r++) {
                    const int ea = a.aexp[(size_t)it.pslot[k] * npad + h0 + row0 + 8 * r];
                    eX[r] = ea == ZERO_EXP ? ZERO_EXP : ea + eAs[k][r];
                }
            }
            for (int i2 = 0; i2 < it.nchild; i2++) {
                if (i2 == i) continue;
                float2 Ev[8][4];
                load_row_block(a.E + ((size_t)(it.pslot[k] * MAXC + i2) * npad + h0 + row0) * 64, t, Ev);
#pragma unroll
                for (int nt = 0; nt < 8; nt++)
#pragma unroll
                    for (int q = 0; q < 4; q++) X[nt][q] = df_mul(X[nt][q], Ev[nt][q]);
            }
            int sh[2];
            bool zero[2];
            normalise_rows<8>(X, NC, sh, zero);
            const size_t eb = (size_t)(it.pslot[k] * MAXC + i);
            store_row_block(a.Ebar + (eb * npad + h0 + row0) * 64, t, X);
            if (t == 0)
#pragma unroll
                for (int r = 0; r < 2; r++)
                    a.ebexp[eb * npad + h0 + row0 + 8 * r] = (zero[r] || eX[r] == ZERO_EXP) ? ZERO_EXP : eX[r] + sh[r];
        }
        if (it.tslot[i][0] < 0) continue;   // tip child: only dlnL/dP
        const bool shared = it.ncls == 1 || it.tslot[i][0] == it.tslot[i][1];
        const int ntarget = shared ? 1 : 2;
        for (int tg = 0; tg < ntarget; tg++) {
            float2 acc[8][4];
            int eacc[2] = {ZERO_EXP, ZERO_EXP};
            const int kbeg = shared ? 0 : tg, kend = shared ? it.ncls : tg + 1;
            for (int k = kbeg; k < kend; k++) {
                const size_t eb = (size_t)(it.pslot[k] * MAXC + i);
                __syncthreads();          // Ebar of this tile is written; previous smem use is over
                slice_tile<NS>(a.Ebar + (eb * npad + h0) * 64, 64, As);
                load_bslices<NS>(a.Bb + (size_t)it.pidx[i][k] * NS * 4096, Bs);
                __syncthreads();
                float2 C[8][4];
                ozaki_mma<NS>(As, Bs, C);
                int eC[2];
#pragma unroll
                for (int r = 0; r < 2; r++) eC[r] = a.ebexp[eb * npad + h0 + row0 + 8 * r];
                if (k == kbeg) {
#pragma unroll
                    for (int nt = 0; nt < 8; nt++)
#pragma unroll
                        for (int q = 0; q < 4; q++) acc[nt][q] = C[nt][q];
                    eacc[0] = eC[0];
                    eacc[1] = eC[1];
                } else {
                    int e[2], da[2], dc[2];
#pragma unroll
                    for (int r = 0; r < 2; r++) {
                        e[r] = max(eacc[r], eC[r]);
                        da[r] = max(eacc[r] - e[r], -1000);
                        dc[r] = max(eC[r] - e[r], -1000);
                    }
#pragma unroll
                    for (int nt = 0; nt < 8; nt++)
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            acc[nt][q] = df_add(df_scale(acc[nt][q], da[q >> 1]), df_scale(C[nt][q], dc[q >> 1]));
                    eacc[0] = e[0];
                    eacc[1] = e[1];
                }
            }
            int sh[2];
            bool zero[2];
            normalise_rows<8>(acc, 64, sh, zero);
            const int ts = it.tslot[i][tg];
            store_row_block(a.Abar + ((size_t)ts * npad + h0 + row0) * 64, t, acc);
            if (t == 0)
#pragma unroll
                for (int r = 0; r < 2; r++)
                    a.aexp[(size_t)ts * npad + h0 + row0 + 8 * r] =
                        (zero[r] || eacc[r] == ZERO_EXP) ? ZERO_EXP : eacc[r] + sh[r];
        }
    }
}

// Partial dlnL/dP of one (branch, omega) pair over a chunk of GCHUNK patterns:
//   G[j][k] = sum_h Ebar[h][j] X[h][k] 2^{x_h},  X = L~ of the child (or one-hot at a tip).
// Internal children: per 64-pattern sub-chunk, A[j][h] = Ebar[h][j] 2^{x_h - xmax}
// and B[k][h] = L~[h][k] as digit planes (transposed), exact tensor-core sums,
// then FP64 accumulation scaled by 2^{xmax}.  Tips: FP64 scatter.
// Warp w owns rows 16 (w & 3) + (0..15) and columns 32 (w >> 2) + (0..31).
template <int NS>
__global__ void __launch_bounds__(256, 1) gradP_fast_kernel(FastBwdArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __nv_bfloat16 *As = reinterpret_cast<__nv_bfloat16 *>(smraw);          // [NS][64][PITCH]
    __nv_bfloat16 *Bs = As + NS * 64 * PITCH;                               // [NS][64][PITCH]
    double *Gs = reinterpret_cast<double *>(Bs + NS * 64 * PITCH);          // [64][65] tip scatter
    int *xs = reinterpret_cast<int *>(Gs + 64 * 65);                        // [64] exponents
    __shared__ int xmax_s;
    const int p = blockIdx.x, chunk = blockIdx.y;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int mrow = (warp & 3) * 16, ncol = (warp >> 2) * 32;
    const size_t npad = a.npad;
    double acc[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[nt][q] = 0.0;
    for (int i = tid; i < 64 * 65; i += 256) Gs[i] = 0.0;
    const int hbeg = chunk * a.gchunk, hend = min(a.npatt, hbeg + a.gchunk);
    for (int ci = a.coff[p]; ci < a.coff[p + 1]; ci++) {
        const Contrib cb = a.contrib[ci];
        for (int hb = hbeg; hb < hend; hb += GSUB) {
            const int nh = min(GSUB, hend - hb);
            __syncthreads();
            if (cb.tslot < 0) {
                if (tid < 64) {
                    const unsigned char *zz = a.z + (size_t)cb.tip * npad + hb;
                    for (int hh = 0; hh < nh; hh++) {
                        const int x = a.ebexp[(size_t)cb.ebar * npad + hb + hh];
                        if (x == ZERO_EXP) continue;
                        const float2 e = a.Ebar[((size_t)cb.ebar * npad + hb + hh) * 64 + tid];
                        Gs[tid * 65 + zz[hh]] += ldexp((double)e.x + (double)e.y, x);
                    }
                }
                continue;
            }
            // exponents of the sub-chunk and their maximum
            if (tid < 64) xs[tid] = tid < nh ? a.ebexp[(size_t)cb.ebar * npad + hb + tid] : ZERO_EXP;
            if (tid == 0) xmax_s = ZERO_EXP;
            __syncthreads();
            if (tid < 64) atomicMax(&xmax_s, xs[tid]);
            __syncthreads();
            const int xmax = xmax_s;
            if (xmax == ZERO_EXP) continue;
            // digit planes, transposed: thread -> pattern pair hp, 8 states s0..s0+7
            {
                const int hp = tid & 31, s0 = (tid >> 5) * 8;
                const int hA = 2 * hp, hB = 2 * hp + 1;
                const int dA = max(xs[hA] - xmax, -1000), dB = max(xs[hB] - xmax, -1000);
                const float2 *eA = a.Ebar + ((size_t)cb.ebar * npad + hb + hA) * 64 + s0;
                const float2 *eB = eA + 64;
                const float2 *lA = a.conP + ((size_t)cb.tslot * npad + hb + hA) * 64 + s0;
                const float2 *lB = lA + 64;
                unsigned *a32 = reinterpret_cast<unsigned *>(As);
                unsigned *b32 = reinterpret_cast<unsigned *>(Bs);
#pragma unroll 2
                for (int u = 0; u < 8; u++) {
                    float d0[NS], d1[NS];
                    const float2 x0 = hA < nh ? df_scale(eA[u], dA) : make_float2(0.f, 0.f);
                    const float2 x1 = hB < nh ? df_scale(eB[u], dB) : make_float2(0.f, 0.f);
                    digits_of<NS>(x0.x, x0.y, d0);
                    digits_of<NS>(x1.x, x1.y, d1);
#pragma unroll
                    for (int s = 0; s < NS; s++) a32[((size_t)s * 64 * PITCH + (s0 + u) * PITCH + hA) >> 1] = bf16x2(d0[s], d1[s]);
                    const float2 y0 = hA < nh ? lA[u] : make_float2(0.f, 0.f);
                    const float2 y1 = hB < nh ? lB[u] : make_float2(0.f, 0.f);
                    digits_of<NS>(y0.x, y0.y, d0);
                    digits_of<NS>(y1.x, y1.y, d1);
#pragma unroll
                    for (int s = 0; s < NS; s++) b32[((size_t)s * 64 * PITCH + (s0 + u) * PITCH + hA) >> 1] = bf16x2(d0[s], d1[s]);
                }
            }
            __syncthreads();
            float2 C[4][4];
            ozaki_mma_block<NS, 4>(As, 64, mrow, Bs, ncol, C);
#pragma unroll
            for (int nt = 0; nt < 4; nt++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[nt][q] += ldexp((double)C[nt][q].x + (double)C[nt][q].y, xmax);
        }
    }
    __syncthreads();
    float2 *out = a.Gpart + ((size_t)p * a.nchunk + chunk) * 64 * 64;
#pragma unroll
    for (int nt = 0; nt < 4; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int j = mrow + g + 8 * (q >> 1);
            const int k = ncol + nt * 8 + 2 * t + (q & 1);
            const double v = acc[nt][q] + Gs[j * 65 + k];
            const float hi = (float)v;
            out[j * 64 + k] = make_float2(hi, (float)(v - (double)hi));
        }
}

template <int NS>
constexpr int gradp_smem() {
    return 2 * NS * 64 * PITCH * 2 + 64 * 65 * 8 + 64 * 4;
}

template <int NS>
cudaError_t init_bwd_ns() {
    cudaError_t e = cudaFuncSetAttribute(bwd_fast_kernel<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, Smem<NS>::BYTES);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(gradP_fast_kernel<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, gradp_smem<NS>());
}

template <int NS>
void launch_bwd_ns(const FastBwdArgs &a, int nitems, int ntile, cudaStream_t st) {
    dim3 grid(ntile, nitems);
    bwd_fast_kernel<NS><<<grid, 256, Smem<NS>::BYTES, st>>>(a);
}

template <int NS>
void launch_gradp_ns(const FastBwdArgs &a, int npair, cudaStream_t st) {
    dim3 grid(npair, a.nchunk);
    gradP_fast_kernel<NS><<<grid, 256, gradp_smem<NS>(), st>>>(a);
}

}  // namespace

cudaError_t init_fast_bwd_kernels(int ns) {
    switch (ns) {
        case 5: return init_bwd_ns<5>();
        case 6: return init_bwd_ns<6>();
        case 7: return init_bwd_ns<7>();
        case 8: return init_bwd_ns<8>();
        default: return cudaErrorInvalidValue;
    }
}

void launch_bwd_fast(const FastBwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st) {
    switch (ns) {
        case 5: launch_bwd_ns<5>(a, nitems, ntile, st); break;
        case 6: launch_bwd_ns<6>(a, nitems, ntile, st); break;
        case 7: launch_bwd_ns<7>(a, nitems, ntile, st); break;
        case 8: launch_bwd_ns<8>(a, nitems, ntile, st); break;
    }
}

void launch_gradP_fast(const FastBwdArgs &a, int ns, int npair, cudaStream_t st) {
    switch (ns) {
        case 5: launch_gradp_ns<5>(a, npair, st); break;
        case 6: launch_gradp_ns<6>(a, npair, st); break;
        case 7: launch_gradp_ns<7>(a, npair, st); break;
        case 8: launch_gradp_ns<8>(a, npair, st); break;
    }
}

}  // namespace gb
