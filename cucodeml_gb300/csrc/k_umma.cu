// tcgen05 versions of the split-precision forward and adjoint-propagation
// kernels (same numerics as k_fast.cu / k_fast_bwd.cu, see there).
//
// Per (128-pattern tile, node, class) CTA and per internal child: the SIMT
// threads cut the child's 128 x 64 double-float tile into NS digit planes
// (K-major core-matrix layout) and copy the NS planes of P; one thread then
// issues, for every significance level L = 2..NS+1, the tcgen05.mma
// (M = 128, N = 64, K = 16, bf16 x bf16 -> FP32) of every digit pair (i, j)
// with i + j = L into that level's 64 TMEM columns (NS = 8: 8 levels = all
// 512 columns), and commits to an mbarrier.  The level sums are exact integers
// in FP32; each thread reads one row (TMEM lane) x 16 columns per level with
// tcgen05.ld and combines the levels in double-float.
// 16 warps (512 threads) per CTA: warp w reads TMEM lanes 32 (w % 4) .. + 31 and
// columns 16 (w / 4) .. + 15, so thread (w, lane) owns pattern row
// 32 (w % 4) + lane and states 16 (w / 4) + 0..15.
// Every mbarrier wait is bounded; on timeout the CTA sets *err, skips its
// remaining work and still frees its TMEM.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include "adjoint_internal.h"
#include "fast_device.cuh"
#include "fast_internal.h"
#include "umma.cuh"

namespace gb {

namespace {

using namespace fastdev;
constexpr int NC = 61;
constexpr int NT = 512;            // threads per CTA
constexpr int NCOL = 16;           // states per thread in the epilogues
constexpr int A_PLANE = 128 * 64 * 2;
constexpr int B_PLANE = 64 * 64 * 2;

template <int NS>
struct USm {
    static constexpr int OFF_B = NS * A_PLANE;
    static constexpr int OFF_MISC = OFF_B + NS * B_PLANE;
    static constexpr int BYTES = OFF_MISC + 16 + 2048 + 4096;   // mbar, tmem slot, row max [4][128], row sums [4][128]
};

// dlnL/dP kernel: A planes of 128 rows (rows 64..127 stay zero), B planes of 64 rows
template <int NB>
struct GSm {
    static constexpr int OFF_B = NB * A_PLANE;
    static constexpr int PLANES = NB * (A_PLANE + B_PLANE);
    static constexpr int OFF_MISC = PLANES > 4 * 4096 * 8 ? PLANES : 4 * 4096 * 8;   // also holds the tip partials
    static constexpr int BYTES = OFF_MISC + 16 + 256 + 64 * 4;  // mbar, tmem slot, exponents, reductions
};

template <int NS>
__device__ __forceinline__ void slice_A_cm(const float2 *__restrict__ src, unsigned char *A) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rr = lane >> 2, kp = lane & 3;
#pragma unroll 2
    for (int q = 0; q < 8; q++) {
        const int cmi = warp * 8 + q;                    // core matrix: row group cmi/8, k group cmi%8
        const int row = (cmi >> 3) * 8 + rr, k = (cmi & 7) * 8 + 2 * kp;
        const float4 v = *reinterpret_cast<const float4 *>(src + (size_t)row * 64 + k);
        int d0[NS], d1[NS];
        digits_of<NS>(v.x, v.y, d0);
        digits_of<NS>(v.z, v.w, d1);
        const int off = cmi * 128 + rr * 16 + kp * 4;
#pragma unroll
        for (int s = 0; s < NS; s++) *reinterpret_cast<unsigned *>(A + s * A_PLANE + off) = bf16_pair(d0[s], d1[s]);
    }
}

// the first NS digit planes of P from global [planes][64][64] (row-major) into core matrices
template <int NS>
__device__ __forceinline__ void load_B_cm(const __nv_bfloat16 *__restrict__ B, unsigned char *Bs) {
    for (int c = threadIdx.x; c < NS * 512; c += blockDim.x) {
        const int s = c >> 9, rem = c & 511, n = rem >> 3, kg = rem & 7;
        const uint4 v = *reinterpret_cast<const uint4 *>(B + (size_t)s * 4096 + n * 64 + kg * 8);
        *reinterpret_cast<uint4 *>(Bs + s * B_PLANE + ((n >> 3) * 8 + kg) * 128 + (n & 7) * 16) = v;
    }
}

// b_top_only: B has a single non-zero digit plane (the first), so only the
// pairs (i, 1) are issued
template <int NS>
__device__ __forceinline__ void issue_levels(uint32_t tmem, uint32_t a_base, uint32_t b_base,
                                             bool b_top_only = false) {
    constexpr uint32_t idesc = umma::make_idesc(128, 64);
#pragma unroll 1
    for (int L = 2; L <= NS + 1; L++) {
        uint32_t acc = 0;
        const int ilo = L - NS > 1 ? L - NS : 1, ihi = L - 1 < NS ? L - 1 : NS;
#pragma unroll 1
        for (int i = ilo; i <= ihi; i++) {
            const int j = L - i;
            if (b_top_only && j != 1) continue;
#pragma unroll
            for (int ks = 0; ks < 4; ks++) {
                const uint64_t ad = umma::make_desc(a_base + (i - 1) * A_PLANE + ks * 256);
                const uint64_t bd = umma::make_desc(b_base + (j - 1) * B_PLANE + ks * 256);
                umma::mma_bf16(tmem + (L - 2) * 64, ad, bd, idesc, acc);
                acc = 1;
            }
        }
    }
}

// All threads: the planes in shared memory are complete (generic-proxy
// stores).  Issue, wait (bounded), read the levels.  Returns a block-uniform
// success flag.
template <int NS>
__device__ __forceinline__ bool contract(unsigned char *sm, uint32_t tmem, uint64_t *mbar, uint32_t &phase,
                                         float2 (&C)[NCOL], int off_b = USm<NS>::OFF_B, bool b_top_only = false) {
    umma::fence_proxy_async();
    umma::fence_before();
    __syncthreads();
    if (threadIdx.x == 0) {
        umma::fence_after();
        issue_levels<NS>(tmem, umma::smem_u32(sm), umma::smem_u32(sm + off_b), b_top_only);
        umma::commit(mbar);
    }
    bool ok = umma::mbar_wait(mbar, phase);
    phase ^= 1u;
    ok = __syncthreads_and(ok);
    umma::fence_after();
    if (ok) {
        const int warp = threadIdx.x >> 5;
        const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
        const int col = NCOL * (warp >> 2);
#pragma unroll
        for (int c = 0; c < NCOL; c++) C[c] = make_float2(0.f, 0.f);
#pragma unroll 1
        for (int L = NS + 1; L >= 2; L--) {
            float v[NCOL];
            umma::tmem_ld16(tmem + lane_base + (L - 2) * 64 + col, v);
            const float w = scalbnf(1.0f, -7 * L);
#pragma unroll
            for (int c = 0; c < NCOL; c++) C[c] = df_add(C[c], make_float2(v[c] * w, 0.f));
        }
    }
    umma::fence_before();
    return ok;
}

__device__ __forceinline__ void load_row32(const float2 *p, float2 (&v)[NCOL]) {
#pragma unroll
    for (int c = 0; c < NCOL / 2; c++) {
        const float4 x = reinterpret_cast<const float4 *>(p)[c];
        v[2 * c] = make_float2(x.x, x.y);
        v[2 * c + 1] = make_float2(x.z, x.w);
    }
}

__device__ __forceinline__ void store_row32(float2 *p, const float2 (&v)[NCOL]) {
#pragma unroll
    for (int c = 0; c < NCOL / 2; c++)
        reinterpret_cast<float4 *>(p)[c] = make_float4(v[2 * c].x, v[2 * c].y, v[2 * c + 1].x, v[2 * c + 1].y);
}

// row maximum over the valid states of the four threads sharing a row
__device__ __forceinline__ float row_max(const float2 (&v)[NCOL], int col0, float *rmax, int row, int ch) {
    float m = 0.f;
#pragma unroll
    for (int c = 0; c < NCOL; c++)
        if (col0 + c < NC) m = fmaxf(m, v[c].x);
    rmax[ch * 128 + row] = m;
    __syncthreads();
    m = fmaxf(fmaxf(rmax[row], rmax[128 + row]), fmaxf(rmax[256 + row], rmax[384 + row]));
    __syncthreads();
    return m;
}

template <int NS>
__global__ void __launch_bounds__(NT, 1) prune_umma_kernel(FastFwdArgs a) {
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + USm<NS>::OFF_MISC);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + USm<NS>::OFF_MISC + 8);
    float *rmax = reinterpret_cast<float *>(sm + USm<NS>::OFF_MISC + 16);
    double *rsum = reinterpret_cast<double *>(sm + USm<NS>::OFF_MISC + 16 + 2048);
    const Item it = a.items[blockIdx.y];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ch = warp >> 2;
    const int row = 32 * (warp & 3) + lane, c0 = NCOL * ch;
    const size_t npad = a.npad;
    const size_t h0 = (size_t)blockIdx.x * 128, h = h0 + row;

    bool internal = false;
    for (int ci = 0; ci < it.nchild; ci++) internal |= it.cslot[ci] >= 0;
    if (internal) {
        if (warp == 0) {
            umma::tmem_alloc(tslot, 512);
            umma::tmem_relinquish();
        }
        if (threadIdx.x == 0) umma::mbar_init(mbar, 1);
        umma::fence_before();
        __syncthreads();
        umma::fence_after();
    }
    const uint32_t tmem = internal ? *tslot : 0u;
    uint32_t phase = 0;
    bool ok = true;
    float2 prod[NCOL];
    int expo = 0;
    for (int ci = 0; ci < it.nchild && ok; ci++) {
        float2 E[NCOL];
        const int cs = it.cslot[ci];
        if (cs < 0) {
            const int zc = a.z[(size_t)it.child[ci] * npad + h];
            load_row32(a.Pdf + (size_t)it.pidx[ci] * 4096 + zc * 64 + c0, E);
        } else {
            __syncthreads();
            slice_A_cm<NS>(a.conP + ((size_t)cs * npad + h0) * 64, sm);
            load_B_cm<NS>(a.Bf + (size_t)it.pidx[ci] * NS * 4096, sm + USm<NS>::OFF_B);
            ok = contract<NS>(sm, tmem, mbar, phase, E);
            if (!ok) break;
            expo += a.expo[(size_t)cs * npad + h];
        }
        if (a.E) store_row32(a.E + ((size_t)(it.eslot + ci) * npad + h) * 64 + c0, E);
#pragma unroll
        for (int c = 0; c < NCOL; c++) prod[c] = ci == 0 ? E[c] : df_mul(prod[c], E[c]);
    }
    if (ok) {
        const float m = row_max(prod, c0, rmax, row, ch);
        const int sh = m > 0.f ? ilogbf(m) + 1 : 0;
        expo += sh;
#pragma unroll
        for (int c = 0; c < NCOL; c++) prod[c] = df_scale(prod[c], -sh);
        if (!it.is_root) {
            store_row32(a.conP + ((size_t)it.slot * npad + h) * 64 + c0, prod);
            if (ch == 0) a.expo[(size_t)it.slot * npad + h] = expo;
        } else {
            double f = 0.0;
#pragma unroll
            for (int c = 0; c < NCOL; c++)
                if (c0 + c < NC) f = fma(a.pi[c0 + c], (double)prod[c].x + (double)prod[c].y, f);
            rsum[ch * 128 + row] = f;
            __syncthreads();
            if (ch == 0) {
                f = (rsum[row] + rsum[128 + row]) + (rsum[256 + row] + rsum[384 + row]);
                if (f <= 0.0) f = 1e-300;
                const double sl = (double)expo * 0.69314718055994530942;
                a.fbar[(size_t)it.cls * npad + h] = f;
                a.ssum[(size_t)it.cls * npad + h] = sl;
                a.fhK[(size_t)it.cls * npad + h] = log(f) + sl;
                a.expo_root[(size_t)it.cls * npad + h] = expo;
            }
        }
    } else if (threadIdx.x == 0) {
        atomicExch(a.err, 1);
        umma::mbar_wait(mbar, phase ^ 1u, 1000000000ull);   // let in-flight MMAs drain (bounded)
    }
    if (internal) {
        umma::fence_before();
        __syncthreads();
        if (warp == 0) umma::tmem_dealloc(tmem, 512);
    }
}

template <int NS>
__global__ void __launch_bounds__(NT, 1) bwd_umma_kernel(FastBwdArgs a) {
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + USm<NS>::OFF_MISC);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + USm<NS>::OFF_MISC + 8);
    float *rmax = reinterpret_cast<float *>(sm + USm<NS>::OFF_MISC + 16);
    const BItem it = a.bitems[blockIdx.y];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ch = warp >> 2;
    const int row = 32 * (warp & 3) + lane, c0 = NCOL * ch;
    const size_t npad = a.npad;
    const size_t h0 = (size_t)blockIdx.x * 128, h = h0 + row;

    bool internal = false;
    for (int i = 0; i < it.nchild; i++) internal |= it.tslot[i][0] >= 0;
    if (internal) {
        if (warp == 0) {
            umma::tmem_alloc(tslot, 512);
            umma::tmem_relinquish();
        }
        if (threadIdx.x == 0) umma::mbar_init(mbar, 1);
        umma::fence_before();
        __syncthreads();
        umma::fence_after();
    }
    const uint32_t tmem = internal ? *tslot : 0u;
    uint32_t phase = 0;
    bool ok = true;

    int eAs[2] = {0, 0};   // exponent of A_a 2^{-sh_a} per class for this row
    for (int k = 0; k < it.ncls; k++) {
        const int c = it.cls[k];
        const int ep = it.is_root ? a.expo_root[(size_t)c * npad + h] : a.expo[(size_t)it.pslot[k] * npad + h];
        int ec = 0;
        for (int i = 0; i < it.nchild; i++)
            if (it.tslot[i][k] >= 0) ec += a.expo[(size_t)it.tslot[i][k] * npad + h];
        eAs[k] = -(ep - ec);
    }

    for (int i = 0; i < it.nchild && ok; i++) {
        for (int k = 0; k < it.ncls; k++) {
            const int c = it.cls[k];
            float2 X[NCOL];
            int eX;
            if (it.is_root) {
                const double g = a.fpatt[h] * a.post[(size_t)c * npad + h] / a.fbar[(size_t)c * npad + h];
#pragma unroll
                for (int q = 0; q < NCOL; q++) {
                    const double v = (c0 + q < NC) ? g * a.pi[c0 + q] : 0.0;
                    const float hi = (float)v;
                    X[q] = make_float2(hi, (float)(v - (double)hi));
                }
                eX = eAs[k];
            } else {
                load_row32(a.Abar + ((size_t)it.pslot[k] * npad + h) * 64 + c0, X);
                const int ea = a.aexp[(size_t)it.pslot[k] * npad + h];
                eX = ea == ZERO_EXP ? ZERO_EXP : ea + eAs[k];
            }
            for (int i2 = 0; i2 < it.nchild; i2++) {
                if (i2 == i) continue;
                float2 Ev[NCOL];
                load_row32(a.E + ((size_t)(it.pslot[k] * MAXC + i2) * npad + h) * 64 + c0, Ev);
#pragma unroll
                for (int q = 0; q < NCOL; q++) X[q] = df_mul(X[q], Ev[q]);
            }
            const float m = row_max(X, c0, rmax, row, ch);
            const int sh = m > 0.f ? ilogbf(m) + 1 : 0;
#pragma unroll
            for (int q = 0; q < NCOL; q++) X[q] = df_scale(X[q], -sh);
            const size_t eb = (size_t)(it.pslot[k] * MAXC + i);
            store_row32(a.Ebar + (eb * npad + h) * 64 + c0, X);
            if (ch == 0) a.ebexp[eb * npad + h] = (!(m > 0.f) || eX == ZERO_EXP) ? ZERO_EXP : eX + sh;
        }
        if (it.tslot[i][0] < 0) continue;
        const bool shared = it.ncls == 1 || it.tslot[i][0] == it.tslot[i][1];
        const int ntarget = shared ? 1 : 2;
        for (int tg = 0; tg < ntarget && ok; tg++) {
            float2 acc[NCOL];
            int eacc = ZERO_EXP;
            const int kbeg = shared ? 0 : tg, kend = shared ? it.ncls : tg + 1;
            for (int k = kbeg; k < kend; k++) {
                const size_t eb = (size_t)(it.pslot[k] * MAXC + i);
                __syncthreads();        // this tile's Ebar rows are written and visible
                slice_A_cm<NS>(a.Ebar + (eb * npad + h0) * 64, sm);
                load_B_cm<NS>(a.Bb + (size_t)it.pidx[i][k] * a.nsP * 4096, sm + USm<NS>::OFF_B);
                float2 C[NCOL];
                ok = contract<NS>(sm, tmem, mbar, phase, C);
                if (!ok) break;
                const int eC = a.ebexp[eb * npad + h];
                if (k == kbeg) {
#pragma unroll
                    for (int q = 0; q < NCOL; q++) acc[q] = C[q];
                    eacc = eC;
                } else {
                    const int e = max(eacc, eC);
                    const int da = max(eacc - e, -1000), dc = max(eC - e, -1000);
#pragma unroll
                    for (int q = 0; q < NCOL; q++) acc[q] = df_add(df_scale(acc[q], da), df_scale(C[q], dc));
                    eacc = e;
                }
            }
            if (!ok) break;
            const float m = row_max(acc, c0, rmax, row, ch);
            const int sh = m > 0.f ? ilogbf(m) + 1 : 0;
#pragma unroll
            for (int q = 0; q < NCOL; q++) acc[q] = df_scale(acc[q], -sh);
            const int ts = it.tslot[i][tg];
            store_row32(a.Abar + ((size_t)ts * npad + h) * 64 + c0, acc);
            if (ch == 0) a.aexp[(size_t)ts * npad + h] = (!(m > 0.f) || eacc == ZERO_EXP) ? ZERO_EXP : eacc + sh;
        }
    }
    if (!ok && threadIdx.x == 0) {
        atomicExch(a.err, 1);
        umma::mbar_wait(mbar, phase ^ 1u, 1000000000ull);   // let in-flight MMAs drain (bounded)
    }
    if (internal) {
        umma::fence_before();
        __syncthreads();
        if (warp == 0) umma::tmem_dealloc(tmem, 512);
    }
}


// Partial dlnL/dP of one (branch, omega) pair over a chunk of patterns (see
// k_fast_bwd.cu for the sums).  Per 64-pattern sub-chunk: A[j][h] =
// Ebar[h][j] 2^{x_h - xmax} and B[k][h] = L~[h][k] (a tip: one-hot at the
// pattern's codon, whose only non-zero digit plane is the first) as digit
// planes with K = patterns; tcgen05 with M = 128 of which rows 64..127 are
// zero; the exact level sums are combined in double-float against a
// reference exponent xr (the chunk's largest), with no FP64 arithmetic until
// the final write.  Threads of TMEM lanes 0..63 (warps w with w % 4 < 2) own
// output rows j, 16 columns each.
template <int NB>
__global__ void __launch_bounds__(NT, 1) gradP_umma_kernel(FastBwdArgs a) {
    extern __shared__ __align__(1024) unsigned char sm[];
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm + GSm<NB>::OFF_MISC);
    uint32_t *tslot = reinterpret_cast<uint32_t *>(sm + GSm<NB>::OFF_MISC + 8);
    int *xs = reinterpret_cast<int *>(sm + GSm<NB>::OFF_MISC + 16);          // [64]
    int *red = reinterpret_cast<int *>(sm + GSm<NB>::OFF_MISC + 16 + 256);   // [2]
    const int p = blockIdx.x, chunk = blockIdx.y;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row = 32 * (warp & 3) + lane, c0 = NCOL * (warp >> 2);
    const size_t npad = a.npad;
    const int hbeg = chunk * a.gchunk, hend = min(a.npatt, hbeg + a.gchunk);
    const int cbeg = a.coff[p], cend = a.coff[p + 1];

    // reference exponent: the largest over the chunk and the pair's contributions
    if (tid == 0) red[0] = ZERO_EXP;
    __syncthreads();
    int xl = ZERO_EXP;
    for (int ci = cbeg; ci < cend; ci++) {
        const int eb = a.contrib[ci].ebar;
        for (int h = hbeg + tid; h < hend; h += NT) xl = max(xl, a.ebexp[(size_t)eb * npad + h]);
    }
    atomicMax(&red[0], xl);
    __syncthreads();
    const int xr = red[0];
    double *out = a.Gpart + ((size_t)p * a.nchunk + chunk) * 64 * 64;
    if (xr == ZERO_EXP) {
        for (int i = tid; i < 4096; i += NT) out[i] = 0.0;
        return;
    }
    if (warp == 0) {
        umma::tmem_alloc(tslot, 512);
        umma::tmem_relinquish();
    }
    if (tid == 0) umma::mbar_init(mbar, 1);
    // A rows 64..127 of every plane stay zero
    for (int i = tid; i < NB * (A_PLANE / 2) / 16; i += NT) {
        const int s = i / (A_PLANE / 2 / 16), r = i % (A_PLANE / 2 / 16);
        reinterpret_cast<uint4 *>(sm + s * A_PLANE + A_PLANE / 2)[r] = make_uint4(0, 0, 0, 0);
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = *tslot;
    uint32_t phase = 0;
    bool ok = true;
    float2 acc[NCOL];
#pragma unroll
    for (int c = 0; c < NCOL; c++) acc[c] = make_float2(0.f, 0.f);
    const int rr = lane >> 2, kp = lane & 3;
    bool any_tip = false;
    for (int ci = cbeg; ci < cend && ok; ci++) {
        const Contrib cb = a.contrib[ci];
        const bool tip = cb.tslot < 0;
        if (tip) {          // one-hot children: segmented scatter below, no digit planes
            any_tip = true;
            continue;
        }
        for (int hb = hbeg; hb < hend && ok; hb += 64) {
            const int nh = min(64, hend - hb);
            __syncthreads();                                   // previous sub-chunk's smem use is over
            if (tid < 64) xs[tid] = tid < nh ? a.ebexp[(size_t)cb.ebar * npad + hb + tid] : ZERO_EXP;
            if (tid == 0) red[1] = ZERO_EXP;
            __syncthreads();
            if (tid < 64) atomicMax(&red[1], xs[tid]);
            __syncthreads();
            const int xmax = red[1];
            if (xmax == ZERO_EXP) continue;
            // transposed digit planes: warp writes core matrices (j group, h group)
            for (int q = 0; q < 4; q++) {
                const int cmi = warp * 4 + q;                  // 64 core matrices: jg = cmi / 8, hg = cmi % 8
                const int j = (cmi >> 3) * 8 + rr, hh = (cmi & 7) * 8 + 2 * kp;
                const int off = cmi * 128 + rr * 16 + kp * 4;
                int d0[NB], d1[NB];
                const float2 *eb = a.Ebar + ((size_t)cb.ebar * npad + hb + hh) * 64 + j;
                const float2 x0 = hh < nh ? df_scale(eb[0], max(xs[hh] - xmax, -1000)) : make_float2(0.f, 0.f);
                const float2 x1 = hh + 1 < nh ? df_scale(eb[64], max(xs[hh + 1] - xmax, -1000)) : make_float2(0.f, 0.f);
                digits_of<NB>(x0.x, x0.y, d0);
                digits_of<NB>(x1.x, x1.y, d1);
#pragma unroll
                for (int s = 0; s < NB; s++) *reinterpret_cast<unsigned *>(sm + s * A_PLANE + off) = bf16_pair(d0[s], d1[s]);
                unsigned char *Bp = sm + GSm<NB>::OFF_B + off;
                if (tip) {
                    const unsigned char *zz = a.z + (size_t)cb.tip * npad + hb;
                    const int z0 = hh < nh ? zz[hh] : -1, z1 = hh + 1 < nh ? zz[hh + 1] : -1;
                    *reinterpret_cast<unsigned *>(Bp) = bf16_pair(z0 == j ? 128 : 0, z1 == j ? 128 : 0);
                } else {
                    const float2 *lb = a.conP + ((size_t)cb.tslot * npad + hb + hh) * 64 + j;
                    const float2 y0 = hh < nh ? lb[0] : make_float2(0.f, 0.f);
                    const float2 y1 = hh + 1 < nh ? lb[64] : make_float2(0.f, 0.f);
                    digits_of<NB>(y0.x, y0.y, d0);
                    digits_of<NB>(y1.x, y1.y, d1);
#pragma unroll
                    for (int s = 0; s < NB; s++) *reinterpret_cast<unsigned *>(Bp + s * B_PLANE) = bf16_pair(d0[s], d1[s]);
                }
            }
            float2 C[NCOL];
            ok = contract<NB>(sm, tmem, mbar, phase, C, GSm<NB>::OFF_B, tip);
            if (!ok) break;
            const int sc = max(xmax - xr, -1000);
#pragma unroll
            for (int c = 0; c < NCOL; c++) acc[c] = df_add(acc[c], df_scale(C[c], sc));
        }
    }
    if (ok && any_tip) {
        // tips: G[j][k] += sum over patterns h with codon z_h = k of Ebar[h][j] 2^{x_h - xr},
        // double-float partial sums in shared memory, 4 pattern partitions x 64 x 64
        __syncthreads();
        float2 *Gt = reinterpret_cast<float2 *>(sm);
        for (int i = tid; i < 4 * 4096; i += NT) Gt[i] = make_float2(0.f, 0.f);
        __syncthreads();
        const int j = tid & 63, part = tid >> 6;
        for (int ci = cbeg; ci < cend && tid < 256; ci++) {
            const Contrib cb = a.contrib[ci];
            if (cb.tslot >= 0) continue;
            const unsigned char *zz = a.z + (size_t)cb.tip * npad;
            const int *xe = a.ebexp + (size_t)cb.ebar * npad;
            const float2 *eb = a.Ebar + (size_t)cb.ebar * npad * 64;
#pragma unroll 4
            for (int hh = hbeg + part; hh < hend; hh += 4) {
                const int x = xe[hh];
                if (x == ZERO_EXP) continue;
                const float2 v = df_scale(eb[(size_t)hh * 64 + j], max(x - xr, -1000));
                float2 *cell = Gt + (part * 64 + zz[hh]) * 64 + j;
                *cell = df_add(*cell, v);
            }
        }
        __syncthreads();
        if (row < 64)
#pragma unroll 4
            for (int c = 0; c < NCOL; c++)
                for (int pp = 0; pp < 4; pp++) acc[c] = df_add(acc[c], Gt[(pp * 64 + c0 + c) * 64 + row]);
    }
    if (ok) {
        if (row < 64)
#pragma unroll
            for (int c = 0; c < NCOL; c++) out[row * 64 + c0 + c] = ldexp((double)acc[c].x + (double)acc[c].y, xr);
    } else if (tid == 0) {
        atomicExch(a.err, 1);
        umma::mbar_wait(mbar, phase ^ 1u, 1000000000ull);
    }
    umma::fence_before();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 512);
}

template <int NS>
cudaError_t init_umma_ns() {
    cudaError_t e = cudaFuncSetAttribute(prune_umma_kernel<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, USm<NS>::BYTES);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(bwd_umma_kernel<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, USm<NS>::BYTES);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(gradP_umma_kernel<NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, GSm<NS>::BYTES);
}

}  // namespace

cudaError_t init_umma_kernels(int ns) {
    switch (ns) {
        case 4: return init_umma_ns<4>();
        case 5: return init_umma_ns<5>();
        case 6: return init_umma_ns<6>();
        case 7: return init_umma_ns<7>();
        case 8: return init_umma_ns<8>();
        default: return cudaErrorInvalidValue;
    }
}

void launch_prune_umma(const FastFwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st) {
    dim3 grid(ntile, nitems);
    switch (ns) {
        case 4: prune_umma_kernel<4><<<grid, NT, USm<4>::BYTES, st>>>(a); break;
        case 5: prune_umma_kernel<5><<<grid, NT, USm<5>::BYTES, st>>>(a); break;
        case 6: prune_umma_kernel<6><<<grid, NT, USm<6>::BYTES, st>>>(a); break;
        case 7: prune_umma_kernel<7><<<grid, NT, USm<7>::BYTES, st>>>(a); break;
        case 8: prune_umma_kernel<8><<<grid, NT, USm<8>::BYTES, st>>>(a); break;
    }
}

void launch_bwd_umma(const FastBwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st) {
    dim3 grid(ntile, nitems);
    switch (ns) {
        case 4: bwd_umma_kernel<4><<<grid, NT, USm<4>::BYTES, st>>>(a); break;
        case 5: bwd_umma_kernel<5><<<grid, NT, USm<5>::BYTES, st>>>(a); break;
        case 6: bwd_umma_kernel<6><<<grid, NT, USm<6>::BYTES, st>>>(a); break;
        case 7: bwd_umma_kernel<7><<<grid, NT, USm<7>::BYTES, st>>>(a); break;
        case 8: bwd_umma_kernel<8><<<grid, NT, USm<8>::BYTES, st>>>(a); break;
    }
}

void launch_gradP_umma(const FastBwdArgs &a, int ns, int npair, cudaStream_t st) {
    dim3 grid(npair, a.nchunk);
    switch (ns) {
        case 4: gradP_umma_kernel<4><<<grid, NT, GSm<4>::BYTES, st>>>(a); break;
        case 5: gradP_umma_kernel<5><<<grid, NT, GSm<5>::BYTES, st>>>(a); break;
        case 6: gradP_umma_kernel<6><<<grid, NT, GSm<6>::BYTES, st>>>(a); break;
        case 7: gradP_umma_kernel<7><<<grid, NT, GSm<7>::BYTES, st>>>(a); break;
        case 8: gradP_umma_kernel<8><<<grid, NT, GSm<8>::BYTES, st>>>(a); break;
    }
}

}  // namespace gb
