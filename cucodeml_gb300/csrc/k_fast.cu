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
//    unsigned 7-bit digits, v ~ sum_i d_i 2^{-7i} (d_i in 0..127, 128 only for
//    v = 1), each held exactly in a bf16 (NS = 8 by default: 56 bits);
//  * digit products d_a d_b summed over K = 64 states and over the pairs of one
//    significance level (i + j = L) stay below NS * 64 * 127 * 128 < 2^24, so the
//    FP32 accumulation of mma.sync m16n8k16 bf16 is exact; levels
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

namespace gb {

namespace {

constexpr int NC = 61;

// ---------------------------------------------------------------- double-float

__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    const float s = __fadd_rn(p, e);
    return make_float2(s, __fsub_rn(e, __fsub_rn(s, p)));
}

// a + b (exact TwoSum of the high parts)
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    const float s = __fadd_rn(a.x, b.x);
    const float bb = __fsub_rn(s, a.x);
    float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
    e = __fadd_rn(e, __fadd_rn(a.y, b.y));
    const float h = __fadd_rn(s, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}

__device__ __forceinline__ float2 df_scale(float2 a, int e) {   // exact 2^e scaling
    return make_float2(scalbnf(a.x, e), scalbnf(a.y, e));
}

// ---------------------------------------------------------------- digits

// Digits of v = hi + lo (a double-float in [0, 1]) in groups of three 7-bit
// digits (21 bits) at a time.  floor(x + y) for a proper double-float equals
// floor(x) unless x is an integer and y < 0; the remainder is renormalised
// with an exact TwoSum before the next group.
__device__ __forceinline__ void df_floor_step(float &x, float &y, float &c) {
    const float fx = floorf(x);
    const bool is_int = fx == x;
    const bool neg = y < 0.f;
    c = (is_int && neg) ? fx - 1.f : fx;
    const float base = is_int ? (neg ? 1.f : 0.f) : __fsub_rn(x, fx);
    const float s = __fadd_rn(base, y);
    const float bb = __fsub_rn(s, base);
    const float e = __fadd_rn(__fsub_rn(base, __fsub_rn(s, bb)), __fsub_rn(y, bb));
    x = s;
    y = e;
}

__device__ __forceinline__ int small_float_to_int(float c) {   // exact for 0 <= c < 2^23
    return __float_as_int(__fadd_rn(c, 8388608.0f)) - 0x4B000000;
}

template <int NS>
__device__ __forceinline__ void digits_of(float hi, float lo, int (&d)[NS]) {
    float x = hi, y = lo;
#pragma unroll
    for (int g0 = 0; g0 < NS; g0 += 3) {
        const int nd = NS - g0 < 3 ? NS - g0 : 3;
        x = scalbnf(x, 7 * nd);
        y = scalbnf(y, 7 * nd);
        float c;
        df_floor_step(x, y, c);
        int ci = small_float_to_int(c < 0.f ? 0.f : c);
#pragma unroll
        for (int q = 0; q < nd; q++) {
            const int sh = 7 * (nd - 1 - q);
            d[g0 + q] = (g0 == 0 && q == 0) ? (ci >> sh) : ((ci >> sh) & 127);   // first may be 128
        }
    }
}

__device__ __forceinline__ float small_int_to_float(int d) {   // exact for 0 <= d < 2^23
    return __fsub_rn(__int_as_float(0x4B000000 | d), 8388608.0f);
}

__device__ __forceinline__ unsigned bf16_pair(int d0, int d1) {
    // integers up to 256 are exact in bf16: the top 16 bits of the float
    const unsigned u0 = __float_as_uint(small_int_to_float(d0)) >> 16;
    const unsigned u1 = __float_as_uint(small_int_to_float(d1)) & 0xffff0000u;
    return u0 | u1;
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// ---------------------------------------------------------------- P slices

// Per pair: Pdf[k][j] = Pt[k][j] as double-float, and the NS digit planes of
//   Bf[s][j][k] = digit s of P[j][k] = Pt[k][j]   (forward:  out[h][j] = sum_k L[h][k] P[j][k])
//   Bb[s][k][j] = digit s of Pt[k][j]            (adjoint:  out[h][k] = sum_j E[h][j] P[j][k])
template <int NS>
__global__ void __launch_bounds__(256) pslice_kernel(const double *__restrict__ Pt, float2 *__restrict__ Pdf,
                                                     __nv_bfloat16 *__restrict__ Bf,
                                                     __nv_bfloat16 *__restrict__ Bb) {
    const int p = blockIdx.x;
    const double *P = Pt + (size_t)p * 4096;
    float2 *D = Pdf + (size_t)p * 4096;
    __nv_bfloat16 *bf = Bf + (size_t)p * NS * 4096;
    __nv_bfloat16 *bb = Bb + (size_t)p * NS * 4096;
    const double S = ldexp(1.0, 7 * NS);
    for (int i = threadIdx.x; i < 4096; i += blockDim.x) {
        const int k = i >> 6, j = i & 63;
        const double v = P[i];                       // Pt[k][j]
        const float hi = (float)v;
        D[i] = make_float2(hi, (float)(v - (double)hi));
        unsigned long long q = v > 0.0 ? (unsigned long long)floor(v * S) : 0ull;
        for (int s = 0; s < NS; s++) {
            const int sh = 7 * (NS - 1 - s);
            const int dgt = s == 0 ? (int)(q >> sh) : (int)((q >> sh) & 127);
            const __nv_bfloat16 b = __float2bfloat16_rn((float)dgt);
            bf[(size_t)s * 4096 + j * 64 + k] = b;
            bb[(size_t)s * 4096 + k * 64 + j] = b;
        }
    }
}

// ---------------------------------------------------------------- contraction core

constexpr int MT = 128;            // patterns per CTA
constexpr int PITCH = 72;          // bf16 per smem row (64 + 8 pad: conflict-free fragments)

template <int NS>
struct Smem {
    static constexpr int A_ELEMS = NS * MT * PITCH;
    static constexpr int B_ELEMS = NS * 64 * PITCH;
    static constexpr int BYTES = (A_ELEMS + B_ELEMS) * 2 + MT * 4 * 2;
};

// Slice a 128 x 64 double-float tile (rows already normalised to [0, 1]) into
// As[s][row][k]; scale_row[row] (if non-null) is an extra exact 2^e per row.
template <int NS>
__device__ __forceinline__ void slice_tile(const float2 *__restrict__ src, int ld, __nv_bfloat16 *As) {
    const int tid = threadIdx.x;
    const int r = tid >> 1;                  // 256 threads: 2 per row
    const int k0 = (tid & 1) * 32;
    const float4 *s4 = reinterpret_cast<const float4 *>(src + (size_t)r * ld + k0);
    unsigned *a32 = reinterpret_cast<unsigned *>(As);
#pragma unroll 4
    for (int q = 0; q < 16; q++) {           // 2 columns per float4
        const float4 v = s4[q];
        int d0[NS], d1[NS];
        digits_of<NS>(v.x, v.y, d0);
        digits_of<NS>(v.z, v.w, d1);
        const int k = k0 + 2 * q;
#pragma unroll
        for (int s = 0; s < NS; s++)
            a32[((size_t)s * MT * PITCH + r * PITCH + k) >> 1] = bf16_pair(d0[s], d1[s]);
    }
}

template <int NS>
__device__ __forceinline__ void load_bslices(const __nv_bfloat16 *__restrict__ B, __nv_bfloat16 *Bs) {
    // global [NS][64][64] -> smem [NS][64][PITCH], 16-byte chunks
    for (int i = threadIdx.x; i < NS * 64 * 8; i += blockDim.x) {
        const int s = i / 512, rem = i % 512, row = rem >> 3, c = rem & 7;
        const uint4 v = reinterpret_cast<const uint4 *>(B + (size_t)s * 4096 + row * 64)[c];
        *reinterpret_cast<uint4 *>(Bs + (size_t)s * 64 * PITCH + row * PITCH + c * 8) = v;
    }
}

// out[nt][0..3] (double-float): the warp's 16 x 64 block of A . B^T over
// K = 64, from the digit planes in shared memory.
template <int NS>
__device__ __forceinline__ void ozaki_mma(const __nv_bfloat16 *As, const __nv_bfloat16 *Bs, float2 (&out)[8][4]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const unsigned *a32 = reinterpret_cast<const unsigned *>(As);
    const unsigned *b32 = reinterpret_cast<const unsigned *>(Bs);
#pragma unroll
    for (int nt = 0; nt < 8; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) out[nt][q] = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int L = NS + 1; L >= 2; L--) {       // smallest significance first
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[nt][q] = 0.f;
        const int ilo = L - NS > 1 ? L - NS : 1, ihi = L - 1 < NS ? L - 1 : NS;
#pragma unroll 1
        for (int i = ilo; i <= ihi; i++) {
            const int j = L - i;
            const unsigned *A = a32 + (((size_t)(i - 1) * MT * PITCH + (warp * 16 + g) * PITCH) >> 1);
            const unsigned *Bp = b32 + (((size_t)(j - 1) * 64 * PITCH + g * PITCH) >> 1);
#pragma unroll
            for (int ks = 0; ks < 4; ks++) {
                const int kw = ks * 8 + t;     // 32-bit word index of k = ks*16 + 2t
                unsigned a[4];
                a[0] = A[kw];
                a[1] = A[kw + 8 * PITCH / 2];
                a[2] = A[kw + 4];
                a[3] = A[kw + 8 * PITCH / 2 + 4];
#pragma unroll
                for (int nt = 0; nt < 8; nt++) {
                    const unsigned *bp = Bp + nt * 8 * PITCH / 2;
                    mma_bf16(acc[nt], a, bp[kw], bp[kw + 4]);
                }
            }
        }
        const float w = scalbnf(1.0f, -7 * L);
#pragma unroll
        for (int nt = 0; nt < 8; nt++)
#pragma unroll
            for (int q = 0; q < 4; q++) out[nt][q] = df_add(out[nt][q], make_float2(acc[nt][q] * w, 0.f));
    }
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
static void launch_fwd_ns(const FastFwdArgs &a, int nitems, int ntile, bool slice, int npair, cudaStream_t st) {
    if (slice) {
        pslice_kernel<NS><<<npair, 256, 0, st>>>(a.Pt64, const_cast<float2 *>(a.Pdf),
                                                 const_cast<__nv_bfloat16 *>(a.Bf), a.Bb);
        return;
    }
    dim3 grid(ntile, nitems);
    prune_fast_kernel<NS><<<grid, 256, Smem<NS>::BYTES, st>>>(a);
}

void launch_pslice(const FastFwdArgs &a, int ns, int npair, cudaStream_t st) {
    switch (ns) {
        case 5: launch_fwd_ns<5>(a, 0, 0, true, npair, st); break;
        case 6: launch_fwd_ns<6>(a, 0, 0, true, npair, st); break;
        case 7: launch_fwd_ns<7>(a, 0, 0, true, npair, st); break;
        case 8: launch_fwd_ns<8>(a, 0, 0, true, npair, st); break;
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
