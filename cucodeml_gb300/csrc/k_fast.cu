// Split-precision forward kernels (GB_PREC_FAST).
//
// Every quantity in the pruning recursion is non-negative (P clamped >= 0,
// tip vectors 0/1, products and sums of those), so the 61x61 contractions can
// be done exactly in integer arithmetic on the tensor cores:
//
//  * operands are kept as double-float pairs (hi + lo, ~48 bits), rows of
//    conditional likelihoods normalised to max in [0.5, 1) with an integer
//    power-of-two exponent per (slot, pattern) carried separately;
//  * at contraction time each operand value v in [0, 1] is cut into NS
//    balanced digits, v ~ sum_i d_i 2^{-7i} (d_i in -128..128, the first in
//    0..128; fast_device.cuh digits_of), each held exactly in a bf16 (NS = 8 by
//    default: 56 bits); P's planes are unsigned 7-bit digits (0..127, 128 only
//    for P = 1);
//  * digit products d_a d_b summed over K = 64 states and over the pairs of one
//    significance level (i + j = L) stay within NS * 64 * 128 * 128 <= 2^23, so
//    the FP32 accumulation of mma.sync m16n8k16 bf16 is exact; levels
//    L = 2..NS+1 are kept (the triangular truncation) and combined in
//    double-float with weights 2^{-7L};
//  * children's messages are multiplied in double-float, each node's rows are
//    renormalised by an exact power of two, and the root sum, log, scale logs
//    and the mixture are FP64.
//
// The result differs from the FP64 recursion by the 7*NS-bit truncation of
// each operand (relative to its row maximum) and the dropped levels.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "internal.h"
#include "fast_internal.h"
#include "batch_internal.h"
#include "fast_device.cuh"

namespace gb {

namespace {

using namespace fastdev;
constexpr int NC = 61;

// ---------------------------------------------------------------- P slices

// element (n, k) of a 64 x 64 plane in the K-major core-matrix layout of the
// tcgen05 operands: 8 x 8 blocks of 128 contiguous bytes, block (n/8, k/8) at
// block index 8 (n/8) + k/8
__device__ __forceinline__ int cm_index(int n, int k) {
    return (((n >> 3) << 3) + (k >> 3)) * 64 + (n & 7) * 8 + (k & 7);
}

// Per pair: Pdf[k][j] = Pt[k][j] as double-float, and the NS digit planes of
//   Bf[s][j][k] = digit s of P[j][k] = Pt[k][j]   (forward:  out[h][j] = sum_k L[h][k] P[j][k])
//   Bb[s][k][j] = digit s of Pt[k][j]            (adjoint:  out[h][k] = sum_j E[h][j] P[j][k])
// row-major planes (cm = 0, mma.sync kernels) or core-matrix planes (cm = 1,
// tcgen05 kernels, copied to shared memory as they are)
// q = floor(v 2^(7 NS)) of an FP64 value of P (P >= 0 after the clamp)
template <int NS>
__device__ __forceinline__ unsigned long long p_fixed(double v) {
    return v > 0.0 ? (unsigned long long)floor(v * ldexp(1.0, 7 * NS)) : 0ull;
}

// the same from the bit fields of v (integer operations only: v = m 2^(e - 1075)
// with the 53-bit significand m, v in [0, 1]), so that the FP64 pipe is not used
template <int NS>
__device__ __forceinline__ unsigned long long p_fixed_bits(double v) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((u >> 52) & 0x7ff);
    if ((u >> 63) || e == 0) return 0ull;                  // negative, zero or subnormal (< 2^-1022)
    const unsigned long long m = (u & 0xfffffffffffffull) | (1ull << 52);
    const int sh = e - 1075 + 7 * NS;
    if (sh >= 0) return m << sh;                           // v <= 1: sh <= 7 NS - 52 (< 11 bits)
    return sh <= -64 ? 0ull : m >> -sh;
}

template <int NS>
__device__ __forceinline__ int p_digit(unsigned long long q, int s) {
    const int sh = 7 * (NS - 1 - s);
    return s == 0 ? (int)(q >> sh) : (int)((q >> sh) & 127);
}

// 8 values' digit s as one 16-byte row of a core matrix (8 bf16)
template <int NS>
__device__ __forceinline__ uint4 p_row(const unsigned long long (&q)[8], int s) {
    return make_uint4(bf16_pair(p_digit<NS>(q[0], s), p_digit<NS>(q[1], s)),
                      bf16_pair(p_digit<NS>(q[2], s), p_digit<NS>(q[3], s)),
                      bf16_pair(p_digit<NS>(q[4], s), p_digit<NS>(q[5], s)),
                      bf16_pair(p_digit<NS>(q[6], s), p_digit<NS>(q[7], s)));
}

template <int NS>
__device__ __forceinline__ void pslice_body(const double *__restrict__ Pt, float2 *__restrict__ Pdf,
                                            __nv_bfloat16 *__restrict__ Bf, __nv_bfloat16 *__restrict__ Bb,
                                            int cm, int p) {
    const double *P = Pt + (size_t)p * 4096;
    float2 *D = Pdf + (size_t)p * 4096;
    __nv_bfloat16 *bf = Bf + (size_t)p * NS * 4096;
    __nv_bfloat16 *bb = Bb + (size_t)p * NS * 4096;
    if (!cm) {     // row-major planes (mma.sync kernels)
        for (int i = threadIdx.x; i < 4096; i += blockDim.x) {
            const int k = i >> 6, j = i & 63;
            const double v = P[i];                       // Pt[k][j]
            const float hi = (float)v;
            D[i] = make_float2(hi, (float)(v - (double)hi));
            const unsigned long long q = p_fixed<NS>(v);
            for (int s = 0; s < NS; s++) {
                const __nv_bfloat16 b = __float2bfloat16_rn((float)p_digit<NS>(q, s));
                bf[(size_t)s * 4096 + j * 64 + k] = b;
                bb[(size_t)s * 4096 + k * 64 + j] = b;
            }
        }
        return;
    }
    // core-matrix planes: P staged in shared memory, then each thread writes
    // whole 16-byte core-matrix rows (8 consecutive K elements) per plane
    __shared__ unsigned long long Ps[64 * 65];           // floor(Pt[k][j] 2^(7 NS)), rows padded
    for (int i = threadIdx.x; i < 4096; i += blockDim.x) {
        const double v = P[i];
        const float hi = (float)v;
        D[i] = make_float2(hi, (float)(v - (double)hi));
        Ps[(i >> 6) * 65 + (i & 63)] = p_fixed_bits<NS>(v);
    }
    __syncthreads();
    for (int u = threadIdx.x; u < 1024; u += blockDim.x) {
        const int n = (u >> 3) & 63, g = u & 7;
        unsigned long long q[8];
        if (u < 512) {         // forward: B[n = j][k], row = 8 consecutive k
#pragma unroll
            for (int t = 0; t < 8; t++) q[t] = Ps[(8 * g + t) * 65 + n];
#pragma unroll
            for (int s = 0; s < NS; s++)
                *reinterpret_cast<uint4 *>(bf + (size_t)s * 4096 + cm_index(n, 8 * g)) = p_row<NS>(q, s);
        } else {               // adjoint: B[n = k][j], row = 8 consecutive j
#pragma unroll
            for (int t = 0; t < 8; t++) q[t] = Ps[n * 65 + 8 * g + t];
#pragma unroll
            for (int s = 0; s < NS; s++)
                *reinterpret_cast<uint4 *>(bb + (size_t)s * 4096 + cm_index(n, 8 * g)) = p_row<NS>(q, s);
        }
    }
}

template <int NS>
__global__ void __launch_bounds__(256) pslice_kernel(const double *__restrict__ Pt, float2 *__restrict__ Pdf,
                                                     __nv_bfloat16 *__restrict__ Bf,
                                                     __nv_bfloat16 *__restrict__ Bb, int cm) {
    pslice_body<NS>(Pt, Pdf, Bf, Bb, cm, blockIdx.x);
}

// many genes in one launch (core-matrix planes, for the tcgen05 kernels)
template <int NS>
__global__ void __launch_bounds__(256) pslice_batched_kernel(const PsliceArgs *__restrict__ args,
                                                             const int2 *__restrict__ map) {
    const int2 g = map[blockIdx.x];
    const PsliceArgs &a = args[g.x];
    pslice_body<NS>(a.Pt64, a.Pdf, a.Bf, a.Bb, 1, g.y);
}

// ---------------------------------------------------------------- forward level

// One CTA per (128-pattern tile, node, class).  Thread (warp w, lane g,t)
// owns rows 16w+g and 16w+g+8 and, per 8-column block nt, columns 8nt+2t, +1:
// out[nt][0..1] -> row 16w+g, out[nt][2..3] -> row 16w+g+8.
template <int NS>
__global__ void __launch_bounds__(256, 1) prune_fast_kernel(FastFwdArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __nv_bfloat16 *As = reinterpret_cast<__nv_bfloat16 *>(smraw);
    __nv_bfloat16 *Bs = As + Smem<NS>::A_ELEMS;
    const Item it = a.items[blockIdx.y];
    const int h0 = blockIdx.x * MT;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int row0 = warp * 16 + g;          // local rows row0 and row0 + 8
    const size_t npad = a.npad;

    float2 prod[8][4];
    int expo[2] = {0, 0};
    for (int ci = 0; ci < it.nchild; ci++) {
        float2 E[8][4];
        const int cs = it.cslot[ci];
        if (cs < 0) {
            const float2 *P = a.Pdf + (size_t)it.pidx[ci] * 4096;
            const unsigned char *zc = a.z + (size_t)it.child[ci] * npad + h0;
            const int z0 = zc[row0], z1 = zc[row0 + 8];
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const float4 v0 = *reinterpret_cast<const float4 *>(P + z0 * 64 + nt * 8 + 2 * t);
                const float4 v1 = *reinterpret_cast<const float4 *>(P + z1 * 64 + nt * 8 + 2 * t);
                E[nt][0] = make_float2(v0.x, v0.y); E[nt][1] = make_float2(v0.z, v0.w);
                E[nt][2] = make_float2(v1.x, v1.y); E[nt][3] = make_float2(v1.z, v1.w);
            }
        } else {
            __syncthreads();                 // previous child's smem use is over
            slice_tile<NS>(a.conP + ((size_t)cs * npad + h0) * 64, 64, As);
            load_bslices<NS>(a.Bf + (size_t)it.pidx[ci] * NS * 4096, Bs);
            __syncthreads();
            ozaki_mma<NS>(As, Bs, E);
            expo[0] += a.expo[(size_t)cs * npad + h0 + row0];
            expo[1] += a.expo[(size_t)cs * npad + h0 + row0 + 8];
        }
        if (a.E) {
            float2 *e0 = a.E + ((size_t)(it.eslot + ci) * npad + h0 + row0) * 64;
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                *reinterpret_cast<float4 *>(e0 + nt * 8 + 2 * t) = make_float4(E[nt][0].x, E[nt][0].y, E[nt][1].x, E[nt][1].y);
                *reinterpret_cast<float4 *>(e0 + 8 * 64 + nt * 8 + 2 * t) = make_float4(E[nt][2].x, E[nt][2].y, E[nt][3].x, E[nt][3].y);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int q = 0; q < 4; q++) prod[nt][q] = ci == 0 ? E[nt][q] : df_mul(prod[nt][q], E[nt][q]);
    }

    // renormalise each row to max in [0.5, 1) by an exact power of two
    int sh[2];
#pragma unroll
    for (int r = 0; r < 2; r++) {
        float m = 0.f;
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int col = nt * 8 + 2 * t + q;
                if (col < NC) m = fmaxf(m, prod[nt][2 * r + q].x);
            }
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
        sh[r] = m > 0.f ? ilogbf(m) + 1 : 0;
        expo[r] += sh[r];
    }
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) prod[nt][q] = df_scale(prod[nt][q], -sh[q >> 1]);

    if (!it.is_root) {
        float2 *o = a.conP + ((size_t)it.slot * npad + h0 + row0) * 64;
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            *reinterpret_cast<float4 *>(o + nt * 8 + 2 * t) = make_float4(prod[nt][0].x, prod[nt][0].y, prod[nt][1].x, prod[nt][1].y);
            *reinterpret_cast<float4 *>(o + 8 * 64 + nt * 8 + 2 * t) = make_float4(prod[nt][2].x, prod[nt][2].y, prod[nt][3].x, prod[nt][3].y);
        }
        if (t == 0) {
            a.expo[(size_t)it.slot * npad + h0 + row0] = expo[0];
            a.expo[(size_t)it.slot * npad + h0 + row0 + 8] = expo[1];
        }
        return;
    }
    // root: f~ = sum_j pi_j L~[h][j] in FP64; log f = log f~ + expo * ln 2
#pragma unroll
    for (int r = 0; r < 2; r++) {
        double f = 0.0;
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int col = nt * 8 + 2 * t + q;
                if (col < NC) {
                    const float2 v = prod[nt][2 * r + q];
                    f = fma(a.pi[col], (double)v.x + (double)v.y, f);
                }
            }
        f += __shfl_xor_sync(0xffffffffu, f, 1);
        f += __shfl_xor_sync(0xffffffffu, f, 2);
        if (t == 0) {
            const size_t h = h0 + row0 + 8 * r;
            if (f <= 0.0) f = 1e-300;
            const double sl = (double)expo[r] * 0.69314718055994530942;
            a.fbar[(size_t)it.cls * npad + h] = f;
            a.ssum[(size_t)it.cls * npad + h] = sl;
            a.fhK[(size_t)it.cls * npad + h] = log(f) + sl;
            a.expo_root[(size_t)it.cls * npad + h] = expo[r];
        }
    }
}

}  // namespace

template <int NS>
static cudaError_t init_ns() {
    return cudaFuncSetAttribute(prune_fast_kernel<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, Smem<NS>::BYTES);
}

cudaError_t init_fast_kernels(int ns) {
    switch (ns) {
        case 5: return init_ns<5>();
        case 6: return init_ns<6>();
        case 7: return init_ns<7>();
        case 8: return init_ns<8>();
        default: return cudaErrorInvalidValue;
    }
}

template <int NS>
static void launch_fwd_ns(const FastFwdArgs &a, int nitems, int ntile, bool slice, int npair, cudaStream_t st,
                          int cm = 0) {
    if (slice) {
        pslice_kernel<NS><<<npair, 256, 0, st>>>(a.Pt64, const_cast<float2 *>(a.Pdf),
                                                 const_cast<__nv_bfloat16 *>(a.Bf), a.Bb, cm);
        return;
    }
    dim3 grid(ntile, nitems);
    prune_fast_kernel<NS><<<grid, 256, Smem<NS>::BYTES, st>>>(a);
}

void launch_pslice(const FastFwdArgs &a, int ns, int npair, bool cm, cudaStream_t st) {
    switch (ns) {
        case 5: launch_fwd_ns<5>(a, 0, 0, true, npair, st, cm); break;
        case 6: launch_fwd_ns<6>(a, 0, 0, true, npair, st, cm); break;
        case 7: launch_fwd_ns<7>(a, 0, 0, true, npair, st, cm); break;
        case 8: launch_fwd_ns<8>(a, 0, 0, true, npair, st, cm); break;
    }
}

void launch_pslice_batched(const PsliceArgs *args, const int2 *map, int nblocks, int ns, cudaStream_t st) {
    if (nblocks <= 0) return;
    switch (ns) {
        case 5: pslice_batched_kernel<5><<<nblocks, 256, 0, st>>>(args, map); break;
        case 6: pslice_batched_kernel<6><<<nblocks, 256, 0, st>>>(args, map); break;
        case 7: pslice_batched_kernel<7><<<nblocks, 256, 0, st>>>(args, map); break;
        case 8: pslice_batched_kernel<8><<<nblocks, 256, 0, st>>>(args, map); break;
    }
}

void launch_prune_fast(const FastFwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st) {
    switch (ns) {
        case 5: launch_fwd_ns<5>(a, nitems, ntile, false, 0, st); break;
        case 6: launch_fwd_ns<6>(a, nitems, ntile, false, 0, st); break;
        case 7: launch_fwd_ns<7>(a, nitems, ntile, false, 0, st); break;
        case 8: launch_fwd_ns<8>(a, nitems, ntile, false, 0, st); break;
    }
}

}  // namespace gb
