// Device helpers of the split-precision kernels: double-float arithmetic,
// 7-bit digit planes, the exact-integer tensor-core contraction (mma.sync
// m16n8k16 bf16 -> FP32) and row renormalisation.  See k_fast.cu for the
// numerical scheme.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>

namespace gb {
namespace fastdev {

constexpr int ZERO_EXP = -(1 << 20);   // exponent of an all-zero row

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

// (s, e) += S w for a power of two w: s <- fl(s + S w) and the exact rounding
// error of that addition (TwoSum) added to e
__device__ __forceinline__ void two_sum_acc(float2 &se, float S, float w) {
    const float t = __fmaf_rn(S, w, se.x);
    const float bb = __fsub_rn(t, se.x);
    const float err = __fadd_rn(__fsub_rn(se.x, __fsub_rn(t, bb)), __fmaf_rn(S, w, -bb));
    se.x = t;
    se.y = __fadd_rn(se.y, err);
}

// (s + e) as a normalised double-float (|e| is small against |s| or s = 0)
__device__ __forceinline__ float2 fast_two_sum(float s, float e) {
    const float h = __fadd_rn(s, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}

// exact 2^e scaling: a multiplication by 2^e built from its exponent bits when
// 2^e is a normal float (the product is then rounded exactly as scalbnf
// rounds it), scalbnf otherwise
__device__ __forceinline__ float2 df_scale(float2 a, int e) {
    if (e >= -126 && e <= 127) {
        const float s = __int_as_float((127 + e) << 23);
        return make_float2(a.x * s, a.y * s);
    }
    return make_float2(scalbnf(a.x, e), scalbnf(a.y, e));
}

// ---------------------------------------------------------------- digits

// Signed digits of v = hi + lo (a double-float, 0 <= v <= 1, |lo| <= ulp(hi)/2):
//   v = sum_s d_s 2^(-7(s+1)) + r,   |r| <= 2^(-7 NS - 1) + 2^-59  (2^(-7 NS) for NS <= 5),
// d_0 in [0, 128], d_s in [-128, 128], every d_s an integer held exactly in a
// bf16.  Each digit is the nearest integer (balanced digits), computed with the
// exact FP32 step  d = rint(128 x) (by the 1.5 2^23 shifter), x <- 128 x - d,
// so every remainder stays within half a unit.  hi gives digits 0..4; lo can
// reach only digits 3 and up (|lo| 2^21 <= 2^-4) and gives its own digits 3
// and 4; where both touch a digit it stays within 128 (hi's part there is at
// most 64, lo's at most 64).  The two remainders (each within half a unit of
// digit 4) are then added in FP32 (rounding error below 2^-59) and digits
// 5..NS-1 come from the sum.
template <int NS>
__device__ __forceinline__ void digits_of(float hi, float lo, float (&d)[NS]) {
    static_assert(NS >= 4, "lo enters at digit 3");
    constexpr int NH = NS < 5 ? NS : 5;
    constexpr float SHIFT = 12582912.0f;      // 1.5 2^23: fl(y + SHIFT) - SHIFT = rint(y), |y| <= 2^22
    float x = hi;
#pragma unroll
    for (int s = 0; s < NH; s++) {
        d[s] = __fsub_rn(__fmaf_rn(x, 128.f, SHIFT), SHIFT);
        x = __fmaf_rn(x, 128.f, -d[s]);
    }
    float w = __fmul_rn(lo, 2097152.0f);       // lo 2^21 (exact)
#pragma unroll
    for (int s = 3; s < NH; s++) {
        const float e = __fsub_rn(__fmaf_rn(w, 128.f, SHIFT), SHIFT);
        w = __fmaf_rn(w, 128.f, -e);
        d[s] = __fadd_rn(d[s], e);
    }
    float r = __fadd_rn(x, w);
#pragma unroll
    for (int s = 5; s < NS; s++) {
        d[s] = __fsub_rn(__fmaf_rn(r, 128.f, SHIFT), SHIFT);
        if (s + 1 < NS) r = __fmaf_rn(r, 128.f, -d[s]);
    }
}

// two integer-valued floats (|d| <= 256) as a bf16 pair, d0 in the low half
__device__ __forceinline__ unsigned bf16x2(float d0, float d1) {
    unsigned u;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(u) : "f"(d1), "f"(d0));
    return u;
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
        float d0[NS], d1[NS];
        digits_of<NS>(v.x, v.y, d0);
        digits_of<NS>(v.z, v.w, d1);
        const int k = k0 + 2 * q;
#pragma unroll
        for (int s = 0; s < NS; s++)
            a32[((size_t)s * MT * PITCH + r * PITCH + k) >> 1] = bf16x2(d0[s], d1[s]);
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

// out[nt][0..3] (double-float): a 16 x (8 NT) block of A . B^T over K = 64
// from the digit planes in shared memory.  A rows a_row0 + (0..15) of planes
// of a_rows rows each; B rows (output columns) n0 + (0..8NT-1).
template <int NS, int NT>
__device__ __forceinline__ void ozaki_mma_block(const __nv_bfloat16 *As, int a_rows, int a_row0,
                                                const __nv_bfloat16 *Bs, int n0, float2 (&out)[NT][4]) {
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3;
    const unsigned *a32 = reinterpret_cast<const unsigned *>(As);
    const unsigned *b32 = reinterpret_cast<const unsigned *>(Bs);
#pragma unroll
    for (int nt = 0; nt < NT; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) out[nt][q] = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int L = NS + 1; L >= 2; L--) {       // smallest significance first
        float acc[NT][4];
#pragma unroll
        for (int nt = 0; nt < NT; nt++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[nt][q] = 0.f;
        const int ilo = L - NS > 1 ? L - NS : 1, ihi = L - 1 < NS ? L - 1 : NS;
#pragma unroll 1
        for (int i = ilo; i <= ihi; i++) {
            const int j = L - i;
            const unsigned *A = a32 + (((size_t)(i - 1) * a_rows * PITCH + (a_row0 + g) * PITCH) >> 1);
            const unsigned *Bp = b32 + (((size_t)(j - 1) * 64 * PITCH + (n0 + g) * PITCH) >> 1);
#pragma unroll
            for (int ks = 0; ks < 4; ks++) {
                const int kw = ks * 8 + t;     // 32-bit word index of k = ks*16 + 2t
                unsigned a[4];
                a[0] = A[kw];
                a[1] = A[kw + 8 * PITCH / 2];
                a[2] = A[kw + 4];
                a[3] = A[kw + 8 * PITCH / 2 + 4];
#pragma unroll
                for (int nt = 0; nt < NT; nt++) {
                    const unsigned *bp = Bp + nt * 8 * PITCH / 2;
                    mma_bf16(acc[nt], a, bp[kw], bp[kw + 4]);
                }
            }
        }
        const float w = scalbnf(1.0f, -7 * L);
#pragma unroll
        for (int nt = 0; nt < NT; nt++)
#pragma unroll
            for (int q = 0; q < 4; q++) out[nt][q] = df_add(out[nt][q], make_float2(acc[nt][q] * w, 0.f));
    }
}

// the warp's 16 x 64 block of a 128-row A tile (forward / adjoint propagation)
template <int NS>
__device__ __forceinline__ void ozaki_mma(const __nv_bfloat16 *As, const __nv_bfloat16 *Bs, float2 (&out)[8][4]) {
    ozaki_mma_block<NS, 8>(As, MT, (threadIdx.x >> 5) * 16, Bs, 0, out);
}

// Renormalise the thread's two rows (out[.][0..1] -> row 0, [2..3] -> row 1,
// columns 8nt + 2t + {0,1}) to max in [0.5, 1) by exact powers of two; the
// four lanes of a quad share rows.  Returns the applied shift per row in sh;
// rows that are all zero get shift 0 and zero[r] = true.
template <int NT>
__device__ __forceinline__ void normalise_rows(float2 (&v)[NT][4], int n_valid, int (&sh)[2], bool (&zero)[2]) {
    const int t = threadIdx.x & 3;
#pragma unroll
    for (int r = 0; r < 2; r++) {
        float m = 0.f;
#pragma unroll
        for (int nt = 0; nt < NT; nt++)
#pragma unroll
            for (int q = 0; q < 2; q++)
                if (nt * 8 + 2 * t + q < n_valid) m = fmaxf(m, v[nt][2 * r + q].x);
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 1));
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, 2));
        zero[r] = !(m > 0.f);
        sh[r] = zero[r] ? 0 : ilogbf(m) + 1;
    }
#pragma unroll
    for (int nt = 0; nt < NT; nt++)
#pragma unroll
        for (int q = 0; q < 4; q++) v[nt][q] = df_scale(v[nt][q], -sh[q >> 1]);
}

}  // namespace fastdev
}  // namespace gb
