// tcgen05 versions of the split-precision kernels (forward, adjoint
// propagation, dlnL/dP; same numerics as k_fast.cu / k_fast_bwd.cu, see there).
//
// Per (128-pattern tile, node, class) task and per internal child: one thread
// starts a bulk copy (cp.async.bulk, completion on an mbarrier) of the NS
// digit planes of P, stored in global memory already in the K-major
// core-matrix layout.  The contraction is warp-specialised and pipelined over
// its four K steps (slice_contract): warps 1..15 cut the child's 128 x 64
// double-float tile into NS digit planes in shared memory step by step and
// arrive on a named barrier per step; warp 0 (one elected lane, descriptors
// from compile-time offsets) issues each step's tcgen05.mma (M = 128, bf16 x
// bf16 -> FP32) as soon as the step is cut and commits to an mbarrier.  Level
// L = 2..NS+1 sums the digit pairs (i, L - i) in TMEM columns 64 (L - 2) (NS =
// 8: all 512 columns); consecutive B planes being contiguous, A plane i against
// B planes j0..j0+3 is one MMA of N = 256 (issue_kstep).  The level sums are
// exact integers in FP32; each thread reads one row (TMEM lane) x NCOL columns
// per level with tcgen05.ld and combines the levels by a compensated sum.
// NWARP warps per CTA: warp w reads TMEM lanes 32 (w % 4) .. + 31 (a warp may
// only access its quarter of the lanes) and columns NCOL (w / 4) .. + NCOL-1,
// so thread (w, lane) owns pattern row 32 (w % 4) + lane and states
// NCOL (w / 4) + 0..NCOL-1.  The adjoint's edge messages use a warp-row layout
// instead (ebar_rows).  dlnL/dP (gradP_task) packs two digit planes per M = 128
// tile and handles tip children as one-hot products.
// Every mbarrier and flag wait is bounded; on timeout the CTA sets *err, lets
// its in-flight MMAs and copies drain (bounded), and still frees its TMEM.
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
constexpr int NT = 512;            // threads per CTA (16 warps; 32 measured no faster)
constexpr int NWARP = NT / 32;
constexpr int NCG = NWARP / 4;     // column groups: warps sharing a TMEM lane quarter
constexpr int NCOL = 64 / NCG;     // states per thread in the epilogues
static_assert(NCOL % 2 == 0 && NWARP == 16, "thread layout: 16 warps, four column groups of 16 states");
constexpr int A_PLANE = 128 * 64 * 2;
constexpr int B_PLANE = 64 * 64 * 2;

// misc block after the planes (struct Misc, 64 B), then the kernel's own
// scratch, the staged argument struct and the staged work item
constexpr int ARGS_BYTES = 256;
constexpr int ITEM_BYTES = 128;
static_assert(sizeof(FastFwdArgs) <= ARGS_BYTES && sizeof(FastBwdArgs) <= ARGS_BYTES, "argument staging");
static_assert(sizeof(Item) <= ITEM_BYTES && sizeof(BItem) <= ITEM_BYTES, "item staging");
// at most one CTA per SM, so that a CTA's 512-column TMEM allocation never waits
constexpr int MIN_SMEM = 120 * 1024;

template <int NS>
struct USm {
    static constexpr int OFF_B = NS * A_PLANE;
    static constexpr int OFF_MISC = OFF_B + NS * B_PLANE;
    static constexpr int OFF_REXP = OFF_MISC + 64;            // int [128] row exponents of a staged tile
    static constexpr int OFF_ARGS = OFF_REXP + 128 * 4;
    static constexpr int OFF_ITEM = OFF_ARGS + 2 * ARGS_BYTES;       // two of each: current and next task
    static constexpr int NEED = OFF_ITEM + 2 * ITEM_BYTES;
    static constexpr int BYTES = NEED > MIN_SMEM ? NEED : MIN_SMEM;
};

// dlnL/dP kernel: digit planes packed 8 KB apart (64 rows x 64 K each), so
// that one M = 128 tile spans two consecutive planes.  Internal children: NB
// planes of Ebar^T then NB of conP; tips: two buffers of NB planes of Ebar^T
// and the one-hot plane.  The task's accumulators G[k][j] (double-float)
// follow, then the usual misc block.
template <int NB>
struct GSm {
    static constexpr int PL = 8192;
    static constexpr int OFF_B = NB * PL;
    static constexpr int INT_BYTES = 2 * NB * PL;
    static constexpr int TIP_BUF = (NB + 1) * PL;
    static constexpr int PLANES = INT_BYTES > 2 * TIP_BUF ? INT_BYTES : 2 * TIP_BUF;
    static constexpr int OFF_ACC = PLANES;
    static constexpr int OFF_MISC = OFF_ACC + 4096 * 8;
    static constexpr int OFF_XS = OFF_MISC + 64;              // int [256] exponents
    static constexpr int OFF_RED = OFF_XS + 1024;             // int [16] reductions
    static constexpr int OFF_ARGS = OFF_RED + 64;
    static constexpr int NEED = OFF_ARGS + ARGS_BYTES;
    static constexpr int BYTES = NEED > MIN_SMEM ? NEED : MIN_SMEM;
};

struct Misc {
    uint64_t mbar;          // MMA completion
    uint64_t mbar_b;        // bulk copy of the P planes (dlnL/dP tips: MMAs of buffer 1)
    uint64_t mstep[4];      // dlnL/dP: MMAs of each K step of a round
    uint32_t tmem;
    int task;
    int okb;                // the P planes arrived (set by the issuing thread)
};
static_assert(sizeof(Misc) <= 64, "misc block");

// cooperative copy of a 4-byte-granular struct into shared memory
template <class T>
__device__ __forceinline__ void stage(T *dst, const T *src) {
    static_assert(sizeof(T) % 4 == 0, "staging granularity");
    for (int i = threadIdx.x; i < (int)(sizeof(T) / 4); i += blockDim.x)
        reinterpret_cast<int *>(dst)[i] = reinterpret_cast<const int *>(src)[i];
}

// ---------------------------------------------------------------- cross-CTA flags

// Wait until *flag == epoch (acquire).  Bounded: gives up after limit_ns
// (2 s unless the handle's wait limit says otherwise), or at once when *err is
// set by another CTA.
__device__ __forceinline__ bool wait_flag(const unsigned *flag, unsigned epoch, const int *err,
                                          uint64_t limit_ns) {
    const uint64_t t0 = umma::global_ns();
    for (int i = 0; i < (1 << 26); i++) {
        unsigned v;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(flag) : "memory");
        if (v == epoch) return true;
        if (*reinterpret_cast<const volatile int *>(err)) return false;
        if (umma::global_ns() - t0 > limit_ns) return false;
        __nanosleep(100);
    }
    return false;
}

// the epoch a consumer waits for and the wait limit, from the control words
__device__ __forceinline__ unsigned wait_epoch(const unsigned *ctl) { return ctl[CTL_EPOCH] + ctl[CTL_SKEW]; }
__device__ __forceinline__ uint64_t wait_limit(const unsigned *ctl) {
    const unsigned ms = ctl[CTL_WAIT_MS];
    return (ms ? ms : 2000u) * 1000000ull;
}

__device__ __forceinline__ void set_flag(unsigned *flag, unsigned epoch) {
    __threadfence();
    asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(flag), "r"(epoch) : "memory");
}

__device__ __forceinline__ unsigned smid() {
    unsigned s;
    asm volatile("mov.u32 %0, %%smid;\n" : "=r"(s));
    return s;
}

// optional task trace, TRACE_WORDS per task: claim time, dependencies met,
// four phase stamps inside the task (0 when absent), end time, SM
enum { TR_CLAIM = 0, TR_READY = 1, TR_P0 = 2, TR_SLICED = 3, TR_MMA = 4, TR_READOUT = 5, TR_END = 6, TR_SM = 7 };
__device__ __forceinline__ void trace_put(unsigned long long *trace, int idx, int slot, unsigned long long v) {
    if (trace && threadIdx.x == 0) trace[(size_t)idx * TRACE_WORDS + slot] = v;
}

// claim the next task index (block-uniform)
__device__ __forceinline__ int claim(unsigned *counter, Misc *m) {
    if (threadIdx.x == 0) m->task = (int)atomicAdd(counter, 1u);
    __syncthreads();
    return m->task;
}

// thread 0: bulk copy of the first NS digit planes of P (global, core-matrix
// layout, 8 KB per plane) into shared memory, completing on m->mbar_b
template <int NS>
__device__ __forceinline__ void start_B(const __nv_bfloat16 *__restrict__ B, unsigned char *Bs, uint64_t *mbar_b) {
    if (threadIdx.x == 0) {
        umma::mbar_expect_tx(mbar_b, NS * B_PLANE);
#pragma unroll
        for (int s = 0; s < NS; s++) umma::bulk_g2s(Bs + s * B_PLANE, B + (size_t)s * 4096, B_PLANE, mbar_b);
    }
}

// Every thread reads its row's NCOL columns of every level and accumulates
//   C = (init ? 0 : C 2^sc_in) + 2^sc_new sum_L S_L 2^(-7L)
// The level sums S_L are exact integers and the weights powers of two: each
// term is added smallest level first with an exact TwoSum into (s, e), the
// rounding errors summed in e (a compensated sum, as accurate as double-float
// additions at 7 instead of 12 FP32 operations), and (s, e) is renormalised
// once at the end.
template <int NS>
__device__ __forceinline__ void readout(Misc *m, float2 (&C)[NCOL], bool init, int sc_in, int sc_new) {
    const int warp = threadIdx.x >> 5;
    const int col = NCOL * (warp >> 2);
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
#pragma unroll
    for (int c = 0; c < NCOL; c++) C[c] = init ? make_float2(0.f, 0.f) : df_scale(C[c], sc_in);
    // two levels per TMEM wait, smallest first
#pragma unroll 1
    for (int L = NS + 1; L >= 2; L -= 2) {
        const int L2 = L - 1 >= 2 ? L - 1 : L;
        uint32_t r0[NCOL], r1[NCOL];
        umma::tmem_ld_nowait(m->tmem + lane_base + (L - 2) * 64 + col, r0);
        umma::tmem_ld_nowait(m->tmem + lane_base + (L2 - 2) * 64 + col, r1);
        umma::tmem_wait_ld();
        const float w0 = scalbnf(1.0f, -7 * L + sc_new);
#pragma unroll
        for (int c = 0; c < NCOL; c++) two_sum_acc(C[c], __uint_as_float(r0[c]), w0);
        if (L2 != L) {
            const float w1 = scalbnf(1.0f, -7 * L2 + sc_new);
#pragma unroll
            for (int c = 0; c < NCOL; c++) two_sum_acc(C[c], __uint_as_float(r1[c]), w1);
        }
    }
#pragma unroll
    for (int c = 0; c < NCOL; c++) C[c] = fast_two_sum(C[c].x, C[c].y);
    umma::fence_before();
}

// ---------------------------------------------------------------- pipelined contractions
//
// Warp-specialised contraction: warps 1..15 cut the operand planes K step by
// K step (16 contraction indices = core-matrix columns 2 KS, 2 KS + 1), taking
// the 32 core matrices of each step round-robin in step-major order
// (n = 32 KS + t, warp 1 + n mod 15); a warp arrives on named barrier 1 + KS
// (after its async-proxy fence) once it has cut its last core matrix of step
// KS, without waiting.  Warp 0 cuts nothing: it waits on each step's barrier
// and issues that step's MMAs, so the tensor pipe works on step KS while the
// other warps cut the next steps, then commits; every thread waits for the
// commit as in mma_round.  Each barrier id completes once per contraction; the
// next contraction's arrivals come after this one's commit wait.
constexpr int CUT_WARPS = NWARP - 1;
constexpr int CUT_MAX = (128 + CUT_WARPS - 1) / CUT_WARPS;     // core matrices per cutting warp, at most

// The MMAs of K step KS for every level: level L = 2..NS+1 sums the digit
// pairs (i, L - i) into TMEM columns 64 (L - 2).  Consecutive B planes are
// contiguous in the K-major core-matrix layout (a plane is 8 row groups of
// 1024 B) and the levels are contiguous in TMEM, so A plane i against B planes
// j0..j0+m-1 is one MMA of N = 64 m (m <= 4) into the columns of levels
// i+j0..i+j0+m-1: 12 MMAs per step for NS = 8 instead of 36 of N = 64, each A
// tile read from shared memory once per up to four B planes.  Plane 1 of A
// meets every level once, so its MMAs of step 0 carry the accumulate flag
// (overwrite the level sums unless accumulating) and all others add.
// Shared-memory descriptor start addresses are in 16-byte units in the low
// 14 bits, so plane and K-step offsets are added to the base descriptors.
template <int NS, int KS>
__device__ __forceinline__ void issue_kstep(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t leader,
                                            uint32_t accumulate) {
#pragma unroll
    for (int i = 1; i <= NS; i++) {
#pragma unroll
        for (int j0 = 1; j0 <= NS + 1 - i; j0 += 4) {
            const int mm = NS + 2 - i - j0 < 4 ? NS + 2 - i - j0 : 4;
            const uint32_t idesc = umma::make_idesc(128, 64 * mm);
            const uint64_t ad = adesc + (uint64_t)(((i - 1) * A_PLANE + KS * 256) >> 4);
            const uint64_t bd = bdesc + (uint64_t)(((j0 - 1) * B_PLANE + KS * 256) >> 4);
            umma::mma_bf16_leader(tmem + (i + j0 - 2) * 64, ad, bd, idesc, (i == 1 && KS == 0) ? accumulate : 1u,
                                  leader);
        }
    }
}

template <int NS, int KS>
__device__ __forceinline__ void issue_step(unsigned char *sm, Misc *m, uint32_t phase, int off_b, bool wait_b,
                                           bool accumulate, bool &okb) {
    umma::bar_sync(1 + KS, NT);
    umma::fence_after();
    if (KS == 0) okb = !wait_b || umma::mbar_wait(&m->mbar_b, phase);
    const uint32_t leader = umma::elect_one();
    if (okb)
        issue_kstep<NS, KS>(m->tmem, umma::make_desc(umma::smem_u32(sm)), umma::make_desc(umma::smem_u32(sm + off_b)),
                            leader, accumulate ? 1u : 0u);
}

// warp 0: issue the four steps as they are cut, then commit
template <int NS>
__device__ __forceinline__ void issue_steps(unsigned char *sm, Misc *m, uint32_t phase, int off_b, bool wait_b,
                                            bool accumulate, unsigned long long *t_cut) {
    bool okb = true;
    issue_step<NS, 0>(sm, m, phase, off_b, wait_b, accumulate, okb);
    issue_step<NS, 1>(sm, m, phase, off_b, wait_b, accumulate, okb);
    issue_step<NS, 2>(sm, m, phase, off_b, wait_b, accumulate, okb);
    issue_step<NS, 3>(sm, m, phase, off_b, wait_b, accumulate, okb);
    if (t_cut && threadIdx.x == 0) *t_cut = umma::global_ns();
    if (umma::elect_one()) {
        umma::commit(&m->mbar);
        m->okb = okb;
    }
}

// cutting warp: core matrix n (step-major) is done; arrive when it was this
// warp's last one of its step
__device__ __forceinline__ void cut_done(int n) {
    if (n + CUT_WARPS >= 32 * ((n >> 5) + 1)) {
        umma::fence_proxy_async();
        umma::fence_before();
        umma::bar_arrive(1 + (n >> 5), NT);
    }
}

// all threads, after the steps: wait (bounded) for the committed MMAs;
// block-uniform success flag
__device__ __forceinline__ bool kstep_finish(Misc *m, uint32_t &phase) {
    bool ok = umma::mbar_wait(&m->mbar, phase);
    umma::fence_after();
    phase ^= 1u;
    return __syncthreads_and(ok) && m->okb;
}

// slice_A_cm and mma_round, warp-specialised and pipelined: the 128 x 64
// double-float tile at src (rows normalised to [0, 1]) is cut into NS planes
// while the MMAs of the steps already cut run.  t_cut (nullable): when the
// last step's MMAs were issued.
template <int NS>
__device__ __forceinline__ bool slice_contract(const float2 *__restrict__ src, unsigned char *sm, Misc *m,
                                               uint32_t &phase, int off_b, bool wait_b,
                                               unsigned long long *t_cut = nullptr) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        issue_steps<NS>(sm, m, phase, off_b, wait_b, false, t_cut);
    } else {
        const int rr = lane >> 2, kp = lane & 3;
        float4 v[CUT_MAX];
#pragma unroll
        for (int u = 0; u < CUT_MAX; u++) {              // all loads in flight first
            const int n = warp - 1 + CUT_WARPS * u, t = n & 31;
            const int g = t >> 1, kg = 2 * (n >> 5) + (t & 1);      // row group, k group
            if (n < 128)
                v[u] = __ldcg(reinterpret_cast<const float4 *>(src + (size_t)(8 * g + rr) * 64 + 8 * kg + 2 * kp));
        }
#pragma unroll
        for (int u = 0; u < CUT_MAX; u++) {
            const int n = warp - 1 + CUT_WARPS * u, t = n & 31;
            if (n >= 128) break;
            const int g = t >> 1, kg = 2 * (n >> 5) + (t & 1);
            float d0[NS], d1[NS];
            digits_of<NS>(v[u].x, v[u].y, d0);
            digits_of<NS>(v[u].z, v[u].w, d1);
            const int off = (8 * g + kg) * 128 + rr * 16 + kp * 4;
#pragma unroll
            for (int s = 0; s < NS; s++) *reinterpret_cast<unsigned *>(sm + s * A_PLANE + off) = bf16x2(d0[s], d1[s]);
            cut_done(n);
        }
    }
    return kstep_finish(m, phase);
}


// Staged tile: after a contraction's MMAs have completed, the plane area
// (free until the next contraction's cut) holds a 128 x 64 double-float tile
// that the read-out wrote thread-per-row, so that the epilogue can run in the
// warp-row layout of tip_rows / ebar_rows (warp w rows 8w..8w+7, lane l states
// 2l, 2l+1): coalesced 512-byte row stores and loads, row maxima by warp
// shuffles.  Rows are padded to TROW float2 (528 B): the 32 rows a read-out
// warp writes at once fall in distinct bank groups, and a staged row is read
// as 512 contiguous bytes.
constexpr int TROW = 66;
constexpr int STAGED_BYTES = 128 * TROW * 8;

__device__ __forceinline__ void stage_rows(unsigned char *sm, const float2 (&v)[NCOL]) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4 *d = reinterpret_cast<float4 *>(reinterpret_cast<float2 *>(sm) + (32 * (warp & 3) + lane) * TROW +
                                           NCOL * (warp >> 2));
#pragma unroll
    for (int q = 0; q < NCOL / 2; q++) d[q] = make_float4(v[2 * q].x, v[2 * q].y, v[2 * q + 1].x, v[2 * q + 1].y);
}

// staged row r: this lane's states 2 lane, 2 lane + 1
__device__ __forceinline__ float4 staged_row(const unsigned char *sm, int r) {
    return reinterpret_cast<const float4 *>(reinterpret_cast<const float2 *>(sm) + r * TROW)[threadIdx.x & 31];
}

__device__ __forceinline__ float4 df_mul4(float4 x, float4 e) {
    const float2 x0 = df_mul(make_float2(x.x, x.y), make_float2(e.x, e.y));
    const float2 x1 = df_mul(make_float2(x.z, x.w), make_float2(e.z, e.w));
    return make_float4(x0.x, x0.y, x1.x, x1.y);
}

// warp-row: maximum of a row over the valid states (all lanes get it)
__device__ __forceinline__ float row_max_w(float4 x) {
    const int lane = threadIdx.x & 31;
    float m = fmaxf(2 * lane < NC ? x.x : 0.f, 2 * lane + 1 < NC ? x.z : 0.f);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    return m;
}

__device__ __forceinline__ float4 df_scale4(float4 x, int e) {
    const float2 x0 = df_scale(make_float2(x.x, x.y), e), x1 = df_scale(make_float2(x.z, x.w), e);
    return make_float4(x0.x, x0.y, x1.x, x1.y);
}

// ---------------------------------------------------------------- forward

__device__ __forceinline__ void tmem_setup(Misc *m) {
    if ((threadIdx.x >> 5) == 0) {
        umma::tmem_alloc(&m->tmem, 512);
        umma::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        umma::mbar_init(&m->mbar, 1);
        umma::mbar_init(&m->mbar_b, 1);
        for (int k = 0; k < 4; k++) umma::mbar_init(&m->mstep[k], 1);
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
}

__device__ __forceinline__ void tmem_teardown(Misc *m) {
    umma::fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 0) umma::tmem_dealloc(m->tmem, 512);
}

// after a failed wait: flag the error and let in-flight MMAs (and, with
// drain_b, the last bulk copy) drain, each wait bounded
__device__ __forceinline__ void on_failure(int *err, Misc *m, uint32_t phase, bool drain_b) {
    if (threadIdx.x == 0) {
        atomicExch(err, 1);
        umma::mbar_wait(&m->mbar, phase ^ 1u, 1000000000ull);
        if (drain_b) umma::mbar_wait(&m->mbar_b, phase ^ 1u, 1000000000ull);
    }
}

// An item whose children are all tips (not the root): the product of the
// tips' rows of P for their codons, renormalised per row, in the warp-row
// layout of ebar_rows (warp w rows 8w..8w+7, lane l states 2l and 2l+1): every
// P row is one coalesced 512-byte gather, every conP row one 512-byte store,
// and the row maxima are warp shuffles (no block barrier).
__device__ __forceinline__ void tip_rows(const FastFwdArgs &a, const Item &it, int tile) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t npad = a.npad;
    const size_t r0 = (size_t)tile * 128 + 8 * warp;
    const size_t hl = r0 + (lane & 7);                 // the row of this lane's codons
    float4 X[8];
    {
        const int zl = a.z[(size_t)it.child[0] * npad + hl];
        const float4 *P = reinterpret_cast<const float4 *>(a.Pdf + (size_t)it.pidx[0] * 4096) + lane;
#pragma unroll
        for (int j = 0; j < 8; j++) X[j] = __ldg(P + 32 * __shfl_sync(0xffffffffu, zl, j));
    }
#pragma unroll 1
    for (int ci = 1; ci < it.nchild; ci++) {
        const int zl = a.z[(size_t)it.child[ci] * npad + hl];
        const float4 *P = reinterpret_cast<const float4 *>(a.Pdf + (size_t)it.pidx[ci] * 4096) + lane;
        float4 E[8];
#pragma unroll
        for (int j = 0; j < 8; j++) E[j] = __ldg(P + 32 * __shfl_sync(0xffffffffu, zl, j));
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float2 x0 = df_mul(make_float2(X[j].x, X[j].y), make_float2(E[j].x, E[j].y));
            const float2 x1 = df_mul(make_float2(X[j].z, X[j].w), make_float2(E[j].z, E[j].w));
            X[j] = make_float4(x0.x, x0.y, x1.x, x1.y);
        }
    }
    float4 *dst = reinterpret_cast<float4 *>(a.conP + ((size_t)it.slot * npad + r0) * 64) + lane;
    int shl = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        float m = fmaxf(2 * lane < NC ? X[j].x : 0.f, 2 * lane + 1 < NC ? X[j].z : 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        const int sh = m > 0.f ? ilogbf(m) + 1 : 0;
        const float2 x0 = df_scale(make_float2(X[j].x, X[j].y), -sh);
        const float2 x1 = df_scale(make_float2(X[j].z, X[j].w), -sh);
        dst[32 * j] = make_float4(x0.x, x0.y, x1.x, x1.y);
        if ((lane & 7) == j) shl = sh;
    }
    if (lane < 8) a.expo[(size_t)it.slot * npad + hl] = shl;
}

// One (node, class) item on one 128-pattern tile.  Needs TMEM when the item
// has an internal child.  The children's product runs in the warp-row layout
// (tip_rows): tip children's rows of P gathered row by row, each internal
// child's contraction read out thread-per-row into the staged tile and taken
// from there row by row.  Returns the block-uniform success flag.
template <int NS>
__device__ bool prune_tile(const FastFwdArgs &a, const Item &it, int tile, unsigned char *sm, Misc *m,
                           uint32_t &phase, unsigned long long *tr = nullptr, int tidx = 0) {
    static_assert(STAGED_BYTES <= USm<NS>::OFF_MISC, "staged tile in the plane area");
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t npad = a.npad;
    const size_t h0 = (size_t)tile * 128, r0 = h0 + 8 * warp;
    const size_t hl = r0 + (lane & 7);                 // the row of this lane's scalars
    bool ok = true;
    if (!it.is_root) {
        bool all_tips = true;
        for (int ci = 0; ci < it.nchild; ci++) all_tips = all_tips && it.cslot[ci] < 0;
        if (all_tips) {
            tip_rows(a, it, tile);
            return true;
        }
    }
    float4 X[8];
    bool have = false;
    int expo = 0;                                      // lanes 0..7: row hl's exponent
    // tip children first: their rows of P for their codons (a tip's edge
    // message, not stored: the adjoint gathers it again)
#pragma unroll 1
    for (int ci = 0; ci < it.nchild; ci++) {
        if (it.cslot[ci] >= 0) continue;
        const int zl = a.z[(size_t)it.child[ci] * npad + hl];
        const float4 *P = reinterpret_cast<const float4 *>(a.Pdf + (size_t)it.pidx[ci] * 4096) + lane;
        float4 E[8];
#pragma unroll
        for (int j = 0; j < 8; j++) E[j] = __ldg(P + 32 * __shfl_sync(0xffffffffu, zl, j));
#pragma unroll
        for (int j = 0; j < 8; j++) X[j] = have ? df_mul4(X[j], E[j]) : E[j];
        have = true;
    }
    trace_put(tr, tidx, TR_P0, umma::global_ns());
    bool first = true;
    for (int ci = 0; ci < it.nchild && ok; ci++) {
        const int cs = it.cslot[ci];
        if (cs < 0) continue;
        __syncthreads();                  // the previous contraction's planes and staged tile are free
        start_B<NS>(a.Bf + (size_t)it.pidx[ci] * NS * 4096, sm + USm<NS>::OFF_B, &m->mbar_b);
        unsigned long long t_cut = 0;
        ok = slice_contract<NS>(a.conP + ((size_t)cs * npad + h0) * 64, sm, m, phase, USm<NS>::OFF_B, true,
                                tr ? &t_cut : nullptr);
        if (first) trace_put(tr, tidx, TR_SLICED, t_cut);
        if (!ok) break;
        if (first) trace_put(tr, tidx, TR_MMA, umma::global_ns());
        {
            float2 E[NCOL];
            readout<NS>(m, E, true, 0, 0);
            stage_rows(sm, E);
        }
        if (first) trace_put(tr, tidx, TR_READOUT, umma::global_ns());
        first = false;
        if (lane < 8) expo += __ldcg(a.expo + (size_t)cs * npad + hl);
        __syncthreads();                                   // the tile is staged
        // edge messages of internal children are kept for the adjoint
        float4 *dE = a.E ? reinterpret_cast<float4 *>(a.E + ((size_t)(it.eslot + ci) * npad + r0) * 64) + lane
                         : nullptr;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float4 e = staged_row(sm, 8 * warp + j);
            if (dE) dE[32 * j] = e;
            X[j] = have ? df_mul4(X[j], e) : e;
        }
        have = true;
    }
    if (!ok) {
        on_failure(a.err, m, phase, true);
        return false;
    }
    // per row: renormalise by a power of two; store, or at the root sum pi L~
    int shl = 0;
    double fl = 0.0;
    float4 *dst = it.is_root ? nullptr : reinterpret_cast<float4 *>(a.conP + ((size_t)it.slot * npad + r0) * 64) + lane;
    const double pi0 = 2 * lane < NC ? a.pi[2 * lane] : 0.0, pi1 = 2 * lane + 1 < NC ? a.pi[2 * lane + 1] : 0.0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const float mx = row_max_w(X[j]);
        const int sh = mx > 0.f ? ilogbf(mx) + 1 : 0;
        const float4 x = df_scale4(X[j], -sh);
        if (dst) {
            dst[32 * j] = x;
        } else {
            double f = fma(pi1, (double)x.z + (double)x.w, pi0 * ((double)x.x + (double)x.y));
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
            if ((lane & 7) == j) fl = f;
        }
        if ((lane & 7) == j) shl = sh;
    }
    if (lane < 8) {
        expo += shl;
        if (!it.is_root) {
            a.expo[(size_t)it.slot * npad + hl] = expo;
        } else {
            const double f = fl <= 0.0 ? 1e-300 : fl;
            const double sl = (double)expo * 0.69314718055994530942;
            a.fbar[(size_t)it.cls * npad + hl] = f;
            a.ssum[(size_t)it.cls * npad + hl] = sl;
            a.fhK[(size_t)it.cls * npad + hl] = log(f) + sl;
            a.expo_root[(size_t)it.cls * npad + hl] = expo;
        }
    }
    return true;
}

// one launch per level: blockIdx.y = item of the level, blockIdx.x = tile
template <int NS>
__global__ void __launch_bounds__(NT, 1) prune_umma_kernel(FastFwdArgs args) {
    extern __shared__ __align__(1024) unsigned char sm[];
    Misc *m = reinterpret_cast<Misc *>(sm + USm<NS>::OFF_MISC);
    FastFwdArgs *a = reinterpret_cast<FastFwdArgs *>(sm + USm<NS>::OFF_ARGS);
    Item *it = reinterpret_cast<Item *>(sm + USm<NS>::OFF_ITEM);
    stage(a, &args);
    stage(it, args.items + blockIdx.y);
    __syncthreads();
    bool internal = false;
    for (int ci = 0; ci < it->nchild; ci++) internal |= it->cslot[ci] >= 0;
    if (internal) tmem_setup(m);
    uint32_t phase = 0;
    prune_tile<NS>(*a, *it, blockIdx.x, sm, m, phase);
    if (internal) tmem_teardown(m);
}

// Persistent forward over a task list (gene, item, tile) in dependency order
// (children before parents).  Each CTA claims tasks from an atomic counter;
// before a task it waits (bounded) for the ready flags of its internal
// children's (slot, tile), and after it publishes its own.  Every dependency
// of a claimed task was claimed earlier by a running CTA, so the waits end.
template <int NS>
__global__ void __launch_bounds__(NT, 1) prune_persist_kernel(const FastFwdArgs *__restrict__ genes,
                                                              const Task *__restrict__ tasks, int ntask,
                                                              unsigned *ctl, unsigned long long *trace) {
    extern __shared__ __align__(1024) unsigned char sm[];
    Misc *m = reinterpret_cast<Misc *>(sm + USm<NS>::OFF_MISC);
    const unsigned epoch = ctl[CTL_EPOCH], awaited = wait_epoch(ctl);
    const uint64_t limit = wait_limit(ctl);
    tmem_setup(m);
    uint32_t phase = 0;
    int idx = claim(ctl + CTL_FWD, m);
    for (int par = 0;; par ^= 1) {
        if (idx >= ntask) break;
        // the following task is claimed now and taken up after this one (its
        // index is posted at this task's last barrier); the task's arguments
        // and item are staged in alternating buffers, so that thread 0 still
        // reads this task's while the others stage the next
        unsigned nxt = 0;
        if (threadIdx.x == 0) nxt = atomicAdd(ctl + CTL_FWD, 1u);
        FastFwdArgs *a = reinterpret_cast<FastFwdArgs *>(sm + USm<NS>::OFF_ARGS + par * ARGS_BYTES);
        Item *it = reinterpret_cast<Item *>(sm + USm<NS>::OFF_ITEM + par * ITEM_BYTES);
        trace_put(trace, idx, TR_CLAIM, umma::global_ns());
        const Task t = tasks[idx];
        stage(a, genes + t.gene);
        stage(it, genes[t.gene].items + t.item);
        __syncthreads();
        int good = 1;
        if (threadIdx.x == 0) {
            // the internal children's tiles towards L2 while their flags are awaited
            // (lines written after the prefetch are updated in L2 as usual)
            for (int ci = 0; ci < it->nchild; ci++)
                if (it->cslot[ci] >= 0)
                    umma::prefetch_l2(a->conP + ((size_t)it->cslot[ci] * a->npad + (size_t)t.tile * 128) * 64,
                                      128 * 64 * sizeof(float2));
            for (int ci = 0; ci < it->nchild && good; ci++)
                if (it->cslot[ci] >= 0)
                    good = wait_flag(a->ready + (size_t)it->cslot[ci] * a->ntile + t.tile, awaited, a->err, limit);
        }
        if (!__syncthreads_and(good)) {
            if (threadIdx.x == 0) atomicExch(a->err, 1);
            break;
        }
        trace_put(trace, idx, TR_READY, umma::global_ns());
        if (!prune_tile<NS>(*a, *it, t.tile, sm, m, phase, trace, idx)) break;
        if (threadIdx.x == 0) m->task = (int)nxt;
        __syncthreads();                                   // the tile's rows are written
        trace_put(trace, idx, TR_END, umma::global_ns());
        trace_put(trace, idx, TR_SM, smid());
        if (threadIdx.x == 0 && !it->is_root) set_flag(a->ready + (size_t)it->slot * a->ntile + t.tile, epoch);
        idx = m->task;
    }
    tmem_teardown(m);
}

// ---------------------------------------------------------------- adjoint propagation

// Ebar rows of child edge i under class k for one 128-pattern tile:
//   Ebar_i = A 2^{-sh_a} prod_{siblings s} E_s
// (A: the node's upper partial, or at the root the seed fpatt post / f~ times
// pi), renormalised per row, with the row exponent in ebexp.  Warp-row
// layout: warp w holds rows 8w..8w+7, lane l states 2l and 2l+1 of each, so
// every row is read and written as 512 contiguous bytes and the row maxima
// come from warp shuffles, with no block barrier.  Lane j < 8 loads the
// per-row scalars (exponents, a tip sibling's codon) of row j.
__device__ __forceinline__ void ebar_rows(const FastBwdArgs &a, const BItem &it, int tile, int i, int k) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t npad = a.npad;
    const size_t r0 = (size_t)tile * 128 + 8 * warp;     // this warp's first row
    const size_t hl = r0 + (lane & 7);                   // the row of this lane's scalars
    const int c = it.cls[k], ps = it.pslot[k];
    // exponent of A 2^{-sh_a}: sh_a = expo_a - sum over children of their expo
    int ea = -(it.is_root ? a.expo_root[(size_t)c * npad + hl] : a.expo[(size_t)ps * npad + hl]);
    for (int q = 0; q < it.nchild; q++)
        if (it.tslot[q][k] >= 0) ea += a.expo[(size_t)it.tslot[q][k] * npad + hl];
    int eX = ea;
    if (!it.is_root) {
        const int ax = __ldcg(a.aexp + (size_t)ps * npad + hl);
        eX = ax == ZERO_EXP ? ZERO_EXP : ax + ea;
    }
    float4 X[8];
    if (it.is_root) {
        const float2 g = a.groot[(size_t)c * npad + hl];
        const float2 p0 = __ldg(a.pidf + 2 * lane), p1 = __ldg(a.pidf + 2 * lane + 1);
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float2 gj = make_float2(__shfl_sync(0xffffffffu, g.x, j), __shfl_sync(0xffffffffu, g.y, j));
            const float2 x0 = df_mul(gj, p0), x1 = df_mul(gj, p1);
            X[j] = make_float4(x0.x, x0.y, x1.x, x1.y);
        }
    } else {
        const float4 *src = reinterpret_cast<const float4 *>(a.Abar + ((size_t)ps * npad + r0) * 64) + lane;
#pragma unroll
        for (int j = 0; j < 8; j++) X[j] = __ldcg(src + 32 * j);
    }
    for (int s = 0; s < it.nchild; s++) {
        if (s == i) continue;
        float4 E[8];
        if (it.tslot[s][k] < 0) {                      // a tip: its message is the row of P for its codon
            const int zl = a.z[(size_t)it.child[s] * npad + hl];
            const float4 *P = reinterpret_cast<const float4 *>(a.Pdf + (size_t)it.pidx[s][k] * 4096) + lane;
#pragma unroll
            for (int j = 0; j < 8; j++) E[j] = __ldcg(P + 32 * __shfl_sync(0xffffffffu, zl, j));
        } else {
            const float4 *src =
                reinterpret_cast<const float4 *>(a.E + ((size_t)(ps * MAXC + s) * npad + r0) * 64) + lane;
#pragma unroll
            for (int j = 0; j < 8; j++) E[j] = __ldcg(src + 32 * j);
        }
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float2 x0 = df_mul(make_float2(X[j].x, X[j].y), make_float2(E[j].x, E[j].y));
            const float2 x1 = df_mul(make_float2(X[j].z, X[j].w), make_float2(E[j].z, E[j].w));
            X[j] = make_float4(x0.x, x0.y, x1.x, x1.y);
        }
    }
    const size_t eb = (size_t)(ps * MAXC + i);
    float4 *dst = reinterpret_cast<float4 *>(a.Ebar + (eb * npad + r0) * 64) + lane;
    int shl = 0;
    float mxl = 0.f;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        float m = fmaxf(2 * lane < NC ? X[j].x : 0.f, 2 * lane + 1 < NC ? X[j].z : 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        const int sh = m > 0.f ? ilogbf(m) + 1 : 0;
        const float2 x0 = df_scale(make_float2(X[j].x, X[j].y), -sh);
        const float2 x1 = df_scale(make_float2(X[j].z, X[j].w), -sh);
        dst[32 * j] = make_float4(x0.x, x0.y, x1.x, x1.y);
        if ((lane & 7) == j) {
            shl = sh;
            mxl = m;
        }
    }
    if (lane < 8) a.ebexp[eb * npad + hl] = (!(mxl > 0.f) || eX == ZERO_EXP) ? ZERO_EXP : eX + shl;
}

template <int NS>
__device__ bool bwd_tile(const FastBwdArgs &a, const BItem &it, int tile, unsigned char *sm, Misc *m,
                         uint32_t &phase, unsigned long long *tr = nullptr, int tidx = 0, int only = -1) {
    static_assert(STAGED_BYTES <= USm<NS>::OFF_MISC, "staged tile in the plane area");
    bool first = true;
    int *rexp = reinterpret_cast<int *>(sm + USm<NS>::OFF_REXP);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = 32 * (warp & 3) + lane;
    const size_t npad = a.npad;
    const size_t h0 = (size_t)tile * 128, h = h0 + row, r0 = h0 + 8 * warp;
    bool ok = true;

    for (int i = 0; i < it.nchild && ok; i++) {
        if (only >= 0 && i != only) continue;
        for (int k = 0; k < it.ncls; k++) ebar_rows(a, it, tile, i, k);
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
                if (first) trace_put(tr, tidx, TR_P0, umma::global_ns());
                start_B<NS>(a.Bb + (size_t)it.pidx[i][k] * a.nsP * 4096, sm + USm<NS>::OFF_B, &m->mbar_b);
                const int eC = a.ebexp[eb * npad + h];
                unsigned long long t_cut = 0;
                ok = slice_contract<NS>(a.Ebar + (eb * npad + h0) * 64, sm, m, phase, USm<NS>::OFF_B, true,
                                        tr ? &t_cut : nullptr);
                if (first) trace_put(tr, tidx, TR_SLICED, t_cut);
                if (!ok) break;
                if (first) trace_put(tr, tidx, TR_MMA, umma::global_ns());
                if (k == kbeg) {
                    readout<NS>(m, acc, true, 0, 0);
                    eacc = eC;
                } else {                                   // acc 2^eacc + C 2^eC on the larger exponent
                    const int e = max(eacc, eC);
                    readout<NS>(m, acc, false, max(eacc - e, -1000), max(eC - e, -1000));
                    eacc = e;
                }
                if (first) trace_put(tr, tidx, TR_READOUT, umma::global_ns());
                first = false;
            }
            if (!ok) break;
            // renormalise and store the child's upper partial in the warp-row
            // layout, from the staged tile
            stage_rows(sm, acc);
            if (warp < 4) rexp[row] = eacc;
            __syncthreads();
            const int ts = it.tslot[i][tg];
            float4 *dst = reinterpret_cast<float4 *>(a.Abar + ((size_t)ts * npad + r0) * 64) + lane;
            int shl = 0;
            float mxl = 0.f;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const float4 x = staged_row(sm, 8 * warp + j);
                const float mx = row_max_w(x);
                const int sh = mx > 0.f ? ilogbf(mx) + 1 : 0;
                dst[32 * j] = df_scale4(x, -sh);
                if ((lane & 7) == j) {
                    shl = sh;
                    mxl = mx;
                }
            }
            if (lane < 8) {
                const int ea = rexp[8 * warp + lane];
                a.aexp[(size_t)ts * npad + r0 + lane] = (!(mxl > 0.f) || ea == ZERO_EXP) ? ZERO_EXP : ea + shl;
            }
        }
    }
    if (!ok) {
        on_failure(a.err, m, phase, true);
        return false;
    }
    return true;
}

template <int NS>
__global__ void __launch_bounds__(NT, 1) bwd_umma_kernel(FastBwdArgs args) {
    extern __shared__ __align__(1024) unsigned char sm[];
    Misc *m = reinterpret_cast<Misc *>(sm + USm<NS>::OFF_MISC);
    FastBwdArgs *a = reinterpret_cast<FastBwdArgs *>(sm + USm<NS>::OFF_ARGS);
    BItem *it = reinterpret_cast<BItem *>(sm + USm<NS>::OFF_ITEM);
    stage(a, &args);
    stage(it, args.bitems + blockIdx.y);
    __syncthreads();
    bool internal = false;
    for (int i = 0; i < it->nchild; i++) internal |= it->tslot[i][0] >= 0;
    if (internal) tmem_setup(m);
    uint32_t phase = 0;
    bwd_tile<NS>(*a, *it, blockIdx.x, sm, m, phase);
    if (internal) tmem_teardown(m);
}

// Persistent adjoint propagation over (gene, backward item, tile) tasks in
// root-first order: a task waits for the upper partials (Abar) of its own
// slots, published by its parent's task, and publishes its children's.
template <int NS>
__global__ void __launch_bounds__(NT, 1) bwd_persist_kernel(const FastBwdArgs *__restrict__ genes,
                                                            const Task *__restrict__ tasks, int ntask,
                                                            unsigned *ctl, unsigned long long *trace) {
    extern __shared__ __align__(1024) unsigned char sm[];
    Misc *m = reinterpret_cast<Misc *>(sm + USm<NS>::OFF_MISC);
    const unsigned epoch = ctl[CTL_EPOCH], awaited = wait_epoch(ctl);
    const uint64_t limit = wait_limit(ctl);
    tmem_setup(m);
    uint32_t phase = 0;
    int idx = claim(ctl + CTL_BWD, m);
    for (int par = 0;; par ^= 1) {
        if (idx >= ntask) break;
        // claimed ahead, alternating staging buffers: as in prune_persist_kernel
        unsigned nxt = 0;
        if (threadIdx.x == 0) nxt = atomicAdd(ctl + CTL_BWD, 1u);
        FastBwdArgs *a = reinterpret_cast<FastBwdArgs *>(sm + USm<NS>::OFF_ARGS + par * ARGS_BYTES);
        BItem *it = reinterpret_cast<BItem *>(sm + USm<NS>::OFF_ITEM + par * ITEM_BYTES);
        trace_put(trace, idx, TR_CLAIM, umma::global_ns());
        const Task t = tasks[idx];
        stage(a, genes + t.gene);
        stage(it, genes[t.gene].bitems + t.item);
        __syncthreads();
        int good = 1;
        if (threadIdx.x == 0) {
            // this task's input tiles towards L2 while the flags are awaited: the
            // upper partials and the internal siblings' edge messages
            const size_t r0 = (size_t)t.tile * 128;
            for (int k = 0; k < it->ncls; k++) {
                const int ps = it->pslot[k];
                if (!it->is_root) umma::prefetch_l2(a->Abar + ((size_t)ps * a->npad + r0) * 64, 128 * 64 * sizeof(float2));
                for (int s = 0; s < it->nchild; s++)
                    if (s != t.edge && it->tslot[s][k] >= 0)
                        umma::prefetch_l2(a->E + ((size_t)(ps * MAXC + s) * a->npad + r0) * 64, 128 * 64 * sizeof(float2));
            }
        }
        if (threadIdx.x == 0 && !it->is_root)
            for (int k = 0; k < it->ncls && good; k++)
                good = wait_flag(a->ready + (size_t)it->pslot[k] * a->ntile + t.tile, awaited, a->err, limit);
        if (!__syncthreads_and(good)) {
            if (threadIdx.x == 0) atomicExch(a->err, 1);
            break;
        }
        trace_put(trace, idx, TR_READY, umma::global_ns());
        if (!bwd_tile<NS>(*a, *it, t.tile, sm, m, phase, trace, idx, t.edge)) break;
        if (threadIdx.x == 0) m->task = (int)nxt;
        __syncthreads();
        trace_put(trace, idx, TR_END, umma::global_ns());
        trace_put(trace, idx, TR_SM, smid());
        // publish the children's slots that received an upper partial (this
        // task's item and arguments stay in their buffers until the task after
        // the next is staged, past barriers that thread 0 reaches after this)
        if (threadIdx.x == 0)
            for (int i = 0; i < it->nchild; i++) {
                if (it->tslot[i][0] < 0 || (t.edge >= 0 && i != t.edge)) continue;
                set_flag(a->ready + (size_t)it->tslot[i][0] * a->ntile + t.tile, epoch);
                if (it->ncls == 2 && it->tslot[i][1] != it->tslot[i][0])
                    set_flag(a->ready + (size_t)it->tslot[i][1] * a->ntile + t.tile, epoch);
            }
        idx = m->task;
    }
    tmem_teardown(m);
}

// ---------------------------------------------------------------- dlnL/dP

// Partial dlnL/dP of one (branch, omega) pair over a chunk of patterns (see
// k_fast_bwd.cu for the sums).  Per 64-pattern sub-chunk: A[j][h] =
// Ebar[h][j] 2^{x_h - xmax} and B[k][h] = L~[h][k] as digit planes with
// K = patterns; tcgen05 with M = 128 of which rows 64..127 are zero; the
// exact level sums are combined in double-float against a reference exponent
// xr (the chunk's largest), with no FP64 arithmetic until the final write.
// Children that are tips (one-hot rows) are summed by a segmented scatter in
// shared memory instead.  Threads of TMEM lanes 0..63 (warps w with
// w % 4 < 2) own output rows j, NCOL columns each.
// per-CTA state of the dlnL/dP kernels across tasks: parities of the next
// completions of m->mbar and m->mbar_b, and the rounds completed on m->mstep
struct GState {
    uint32_t phase = 0, phase_b = 0, nround = 0;
};

// read-out partials of the two TMEM lane halves (lanes 0..63: warps 0, 1 of
// each group of four; lanes 64..127: warps 2, 3) for the same G[j][c0..c0+15]:
// added into accs[k][j] one half after the other
__device__ __forceinline__ void combine_halves(float2 *accs, const float2 (&part)[NCOL], int half, int c0, int j) {
    for (int hp = 0; hp < 2; hp++) {
        if (half == hp)
#pragma unroll
            for (int c = 0; c < NCOL; c++) {
                float2 *cell = accs + (c0 + c) * 64 + j;
                *cell = df_add(*cell, fast_two_sum(part[c].x, part[c].y));
            }
        __syncthreads();
    }
}

// dlnL/dP of a pair whose child is a tip:
//   G[j][k] += sum over the chunk's patterns h with the tip's codon z_h = k of Ebar[h][j] 2^{x_h - xr}
// as tensor-core products A B: A = Ebar^T cut into NB digit planes (M = j,
// K = h), packed so that one M = 128 tile holds planes 2m (rows 0..63) and
// 2m + 1 (rows 64..127); B = the one-hot codon matrix of the round's 64
// patterns (exact 0/1, one plane).  D block m (TMEM columns 64 m) accumulates
// planes 2m and 2m + 1 over every 64-pattern round of the chunk and every
// contribution (|sums| <= contributions x gchunk x 128 < 2^24, exact) and is
// read out once.  Rounds alternate between two shared-memory buffers: warps
// 1..15 load round r, wait until the MMAs of round r - 2 are done (committed
// to m->mbar for buffer 0, m->mbar_b for buffer 1), cut, and arrive on named
// barrier 1 + r mod 2; warp 0 issues.  The read-out adds G 2^-xr into accs.
template <int NB>
__device__ bool gradP_tips(const FastBwdArgs &a, int cbeg, int cend, int hbeg, int hend, int xr, unsigned char *sm,
                           Misc *m, GState &gs, float2 *accs) {
    constexpr int NBP = (NB + 1) / 2;              // plane pairs = D blocks
    constexpr int PL = GSm<NB>::PL, TBUF = GSm<NB>::TIP_BUF;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int rr = lane >> 2, kp = lane & 3;
    const size_t npad = a.npad;
    const uint32_t q0 = gs.phase & 1u, q1 = gs.phase_b & 1u;   // parities of the barriers' next completions
    int r = 0;
    bool ok = true;
    for (int ci = cbeg; ci < cend; ci++) {
        const Contrib cb = a.contrib[ci];
        const unsigned char *zz = a.z + (size_t)cb.tip * npad;
        const int *xe = a.ebexp + (size_t)cb.ebar * npad;
        const float2 *eb = a.Ebar + (size_t)cb.ebar * npad * 64;
        if (tid == 32) {                                   // the chunk's rows and exponents towards L2
            umma::prefetch_l2(eb + (size_t)hbeg * 64, (uint32_t)(hend - hbeg) * 64 * sizeof(float2));
            const uint32_t xb = (uint32_t)((hend - hbeg) * sizeof(int)) & ~15u;   // whole 16-byte units only
            if (xb) umma::prefetch_l2(xe + hbeg, xb);
        }
        for (int hs = hbeg; hs < hend; hs += 64, r++) {
            const int b = r & 1, nh = min(64, hend - hs);
            unsigned char *buf = sm + b * TBUF;
            uint64_t *bar = b ? &m->mbar_b : &m->mbar;
            if (warp == 0) {
                umma::bar_sync(1 + b, NT);
                umma::fence_after();
                const uint32_t leader = umma::elect_one();
                constexpr uint32_t idesc = umma::make_idesc(128, 64);
                const uint64_t ad = umma::make_desc(umma::smem_u32(buf));
                const uint64_t bd = umma::make_desc(umma::smem_u32(buf + NB * PL));
#pragma unroll
                for (int ks = 0; ks < 4; ks++)
#pragma unroll
                    for (int mm = 0; mm < NBP; mm++)
                        umma::mma_bf16_leader(m->tmem + 64 * mm, ad + (uint64_t)((2 * mm * PL + ks * 256) >> 4),
                                              bd + (uint64_t)((ks * 256) >> 4), idesc, (r > 0 || ks > 0) ? 1u : 0u,
                                              leader);
                if (leader) umma::commit(bar);
                continue;
            }
            // A: 64 core matrices (j group n / 8, h group n % 8), round-robin over warps 1..15;
            // loads first, then the wait for the buffer
            float2 v[5][2];
            int x[5][2];
#pragma unroll
            for (int u = 0; u < 5; u++) {
                const int n = warp - 1 + CUT_WARPS * u;
                const int j = (n >> 3) * 8 + rr, hh = (n & 7) * 8 + 2 * kp;
                const bool in0 = n < 64 && hh < nh, in1 = n < 64 && hh + 1 < nh;
                v[u][0] = in0 ? __ldcg(eb + (size_t)(hs + hh) * 64 + j) : make_float2(0.f, 0.f);
                v[u][1] = in1 ? __ldcg(eb + (size_t)(hs + hh + 1) * 64 + j) : make_float2(0.f, 0.f);
                x[u][0] = in0 ? __ldcg(xe + hs + hh) : ZERO_EXP;
                x[u][1] = in1 ? __ldcg(xe + hs + hh + 1) : ZERO_EXP;
            }
            const int tb = tid - 32;                        // B rows of this thread: tb and tb + 480 (< 512)
            const uint2 zb0 = *reinterpret_cast<const uint2 *>(zz + hs + 8 * (tb >> 6));
            const uint2 zb1 = tb + (NT - 32) < 512 ? *reinterpret_cast<const uint2 *>(zz + hs + 8 * ((tb + NT - 32) >> 6))
                                                  : make_uint2(0xffffffffu, 0xffffffffu);
            if (r >= 2) ok = umma::mbar_wait(bar, ((b ? q1 : q0) + ((r - 2) >> 1)) & 1u) && ok;
#pragma unroll
            for (int u = 0; u < 5; u++) {
                const int n = warp - 1 + CUT_WARPS * u;
                if (n >= 64) break;
                const float2 y0 = df_scale(v[u][0], max(x[u][0] - xr, -1000));
                const float2 y1 = df_scale(v[u][1], max(x[u][1] - xr, -1000));
                float d0[NB], d1[NB];
                digits_of<NB>(y0.x, y0.y, d0);
                digits_of<NB>(y1.x, y1.y, d1);
                const int off = n * 128 + rr * 16 + kp * 4;
#pragma unroll
                for (int s2 = 0; s2 < NB; s2++)
                    *reinterpret_cast<unsigned *>(buf + s2 * PL + off) = bf16x2(d0[s2], d1[s2]);
            }
            // B: 512 16-byte rows (codon n = row mod 64, pattern group row / 64): 1.0 where z_h = n
            for (int q2 = 0; q2 < 2; q2++) {
                const int t = tb + q2 * (NT - 32);
                if (t >= 512) break;
                const int n = t & 63, kg = t >> 6;
                const uint2 zb = q2 ? zb1 : zb0;
                unsigned w[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const unsigned zw = q < 2 ? zb.x : zb.y, sh = 16 * (q & 1);
                    const unsigned b0 = (zw >> sh) & 255u, b1 = (zw >> (sh + 8)) & 255u;
                    w[q] = (b0 == (unsigned)n ? 0x3F80u : 0u) | (b1 == (unsigned)n ? 0x3F800000u : 0u);
                }
                *reinterpret_cast<uint4 *>(buf + NB * PL + ((n >> 3) * 8 + kg) * 128 + (n & 7) * 16) =
                    make_uint4(w[0], w[1], w[2], w[3]);
            }
            umma::fence_proxy_async();
            umma::fence_before();
            umma::bar_arrive(1 + b, NT);
        }
    }
    // the last two rounds' MMAs (a commit completes after every earlier MMA of its thread)
    for (int rl = r - 2 > 0 ? r - 2 : 0; rl < r; rl++) {
        const int bl = rl & 1;
        ok = umma::mbar_wait(bl ? &m->mbar_b : &m->mbar, ((bl ? q1 : q0) + (rl >> 1)) & 1u) && ok;
    }
    umma::fence_after();
    if (((r + 1) >> 1) & 1) gs.phase ^= 1u;        // rounds on buffer 0: (r + 1) / 2, on buffer 1: r / 2
    if ((r >> 1) & 1) gs.phase_b ^= 1u;
    if (!__syncthreads_and(ok)) return false;
    const int qd = warp & 3, half = qd >> 1, j = 32 * (qd & 1) + lane, c0 = NCOL * (warp >> 2);
    const uint32_t lane_base = (uint32_t)(32 * qd) << 16;
    float2 part[NCOL];
#pragma unroll
    for (int c = 0; c < NCOL; c++) part[c] = make_float2(0.f, 0.f);
#pragma unroll 1
    for (int mm = NBP - 1; mm >= 0; mm -= 2) {     // smallest first, two blocks per TMEM wait
        const int m2 = mm > 0 ? mm - 1 : mm;
        const int sp = 2 * mm + half, sp2 = 2 * m2 + half;
        uint32_t rv[NCOL], rv2[NCOL];
        umma::tmem_ld_nowait(m->tmem + lane_base + 64 * mm + c0, rv);
        umma::tmem_ld_nowait(m->tmem + lane_base + 64 * m2 + c0, rv2);
        umma::tmem_wait_ld();
        if (sp < NB) {                             // (not the rows 64..127 of an odd last pair)
            const float w = scalbnf(1.0f, -7 * (sp + 1));
#pragma unroll
            for (int c = 0; c < NCOL; c++) two_sum_acc(part[c], __uint_as_float(rv[c]), w);
        }
        if (m2 != mm && sp2 < NB) {
            const float w = scalbnf(1.0f, -7 * (sp2 + 1));
#pragma unroll
            for (int c = 0; c < NCOL; c++) two_sum_acc(part[c], __uint_as_float(rv2[c]), w);
        }
    }
    umma::fence_before();
    combine_halves(accs, part, half, c0, j);
    return true;
}

// One K step of an internal child's round: A = Ebar^T planes packed (tile m
// = planes 2m, 2m + 1 in rows 0..63 / 64..127), B = conP planes (K-major,
// consecutive planes contiguous).  Tile m against B planes j0..j0+c-1 is one
// MMA of N = 64 c into TMEM blocks beta = 2m + j0 - 1 .. (block beta: level
// beta + 2 in lanes 0..63, level beta + 3 in lanes 64..127).  Every pair
// (i, j) with i + j <= NB + 1 is covered (for even i also j = NB + 2 - i:
// level NB + 2, not read); tile 0 covers every block, so its step-0 MMAs of
// a block's first round overwrite.  With NB odd the last tile's rows
// 64..127 are the first conP plane (finite, feeding only level NB + 2).
template <int NB, int KS>
__device__ __forceinline__ void issue_int_step(unsigned char *sm, Misc *m, bool first) {
    umma::bar_sync(1 + KS, NT);
    umma::fence_after();
    const uint32_t leader = umma::elect_one();
    const uint64_t adesc = umma::make_desc(umma::smem_u32(sm));
    const uint64_t bdesc = umma::make_desc(umma::smem_u32(sm + GSm<NB>::OFF_B));
#pragma unroll
    for (int mm = 0; mm <= (NB - 1) / 2; mm++) {
#pragma unroll
        for (int j0 = 1; j0 <= NB - 2 * mm; j0 += 4) {
            const int cnt = NB - 2 * mm - j0 + 1 < 4 ? NB - 2 * mm - j0 + 1 : 4;
            const uint32_t idesc = umma::make_idesc(128, 64 * cnt);
            const uint64_t ad = adesc + (uint64_t)((2 * mm * GSm<NB>::PL + KS * 256) >> 4);
            const uint64_t bd = bdesc + (uint64_t)(((j0 - 1) * GSm<NB>::PL + KS * 256) >> 4);
            umma::mma_bf16_leader(m->tmem + (2 * mm + j0 - 1) * 64, ad, bd, idesc,
                                  (mm == 0 && KS == 0 && first) ? 0u : 1u, leader);
        }
    }
    if (leader) umma::commit(&m->mstep[KS]);
}

template <int NB>
__device__ bool gradP_task(const FastBwdArgs &a, int p, int chunk, unsigned char *sm, Misc *m, GState &gs,
                           unsigned long long *tr = nullptr, int tidx = 0) {
    // tracing only: time spent per phase (exponents, -, operand planes with
    // their pipelined MMAs, read-outs), measured by thread 0 between block barriers
    unsigned long long tlast = tr ? umma::global_ns() : 0, tdur[4] = {0, 0, 0, 0};
    auto tick = [&](int slot) {
        if (!tr) return;
        __syncthreads();
        if (threadIdx.x == 0) {
            const unsigned long long now = umma::global_ns();
            tdur[slot] += now - tlast;
            tlast = now;
        }
    };
    int *xs = reinterpret_cast<int *>(sm + GSm<NB>::OFF_XS);
    int *red = reinterpret_cast<int *>(sm + GSm<NB>::OFF_RED);
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
    tick(0);
    float2 *out = a.Gpart + ((size_t)p * a.nchunk + chunk) * 64 * 64;
    if (xr == ZERO_EXP) {
        for (int i = tid; i < 4096; i += NT) out[i] = make_float2(0.f, 0.f);
        return true;
    }
    // the accumulators wait in shared memory between read-outs (thread (row, c0..c0+15)
    // owns G[c0 + c][row], row < 64), so the cutting warps have their registers
    float2 *accs = reinterpret_cast<float2 *>(sm + GSm<NB>::OFF_ACC);
    if (row < 64)
#pragma unroll
        for (int c = 0; c < NCOL; c++) accs[(c0 + c) * 64 + row] = make_float2(0.f, 0.f);
    __syncthreads();
    // the contributions of a pair share its child: all tips or all internal
    if (a.contrib[cbeg].tslot < 0) {
        if (!gradP_tips<NB>(a, cbeg, cend, hbeg, hend, xr, sm, m, gs, accs)) {
            if (tid == 0) {
                atomicExch(a.err, 1);
                umma::mbar_wait(&m->mbar, gs.phase ^ 1u, 1000000000ull);
                umma::mbar_wait(&m->mbar_b, gs.phase_b ^ 1u, 1000000000ull);
            }
            return false;
        }
        tick(2);
    } else {
        // Internal children: per block of 256 patterns (rows scaled against the
        // block's largest exponent), four rounds of 64 add into the same level
        // sums (each TMEM lane half holds at most 4 digit pairs of a level:
        // <= 4 x 256 x 128^2 = 2^24, exact in FP32).  Warps 1..15 cut
        // a round's 128 core matrices step-major (n = 32 KS + t; t < 16: Ebar's,
        // else conP's; j group (t mod 16) / 2, h group 2 KS + t mod 2), each step
        // after that step's MMAs of the previous round are done (m->mstep[KS]),
        // and arrive on named barrier 1 + KS; warp 0 issues each step.
        const int rr = lane >> 2, kp = lane & 3;
        bool ok = true;
        for (int ci = cbeg; ci < cend && ok; ci++) {
            const Contrib cb = a.contrib[ci];
            if (tid == 32) {                               // the chunk's rows towards L2
                const uint32_t bytes = (uint32_t)(hend - hbeg) * 64 * sizeof(float2);
                umma::prefetch_l2(a.Ebar + ((size_t)cb.ebar * npad + hbeg) * 64, bytes);
                umma::prefetch_l2(a.conP + ((size_t)cb.tslot * npad + hbeg) * 64, bytes);
            }
            for (int hb = hbeg; hb < hend && ok; hb += 256) {
                __syncthreads();                               // previous read-out and exponents are done
                if (tid < 256) {                               // warps 0..7: exponents and their maximum
                    const int x = hb + tid < hend ? a.ebexp[(size_t)cb.ebar * npad + hb + tid] : ZERO_EXP;
                    xs[tid] = x;
                    int mx = x;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                    if (lane == 0) red[4 + warp] = mx;
                }
                __syncthreads();
                int xmax = red[4];
#pragma unroll
                for (int q = 5; q < 12; q++) xmax = max(xmax, red[q]);
                tick(0);
                if (xmax == ZERO_EXP) continue;
                for (int half = 0; half < 4; half++) {
                    const int hs = hb + 64 * half, nh = min(64, hend - hs);
                    if (nh <= 0) break;
                    const uint32_t g = gs.nround++;            // this round's index on m->mstep
                    if (warp == 0) {
                        issue_int_step<NB, 0>(sm, m, half == 0);
                        issue_int_step<NB, 1>(sm, m, half == 0);
                        issue_int_step<NB, 2>(sm, m, half == 0);
                        issue_int_step<NB, 3>(sm, m, half == 0);
                        continue;
                    }
                    const int *xh = xs + 64 * half;
                    float2 w0[CUT_MAX], w1[CUT_MAX];
#pragma unroll
                    for (int u = 0; u < CUT_MAX; u++) {         // all loads in flight first
                        const int n = warp - 1 + CUT_WARPS * u, t = n & 31;
                        const int j = ((t & 15) >> 1) * 8 + rr, hh = (2 * (n >> 5) + (t & 1)) * 8 + 2 * kp;
                        const float2 *src = t < 16 ? a.Ebar + ((size_t)cb.ebar * npad + hs + hh) * 64 + j
                                                   : a.conP + ((size_t)cb.tslot * npad + hs + hh) * 64 + j;
                        const float2 z = make_float2(0.f, 0.f);
                        w0[u] = n < 128 && hh < nh ? src[0] : z;
                        w1[u] = n < 128 && hh + 1 < nh ? src[64] : z;
                    }
#pragma unroll
                    for (int u = 0; u < CUT_MAX; u++) {
                        const int n = warp - 1 + CUT_WARPS * u, t = n & 31, ks = n >> 5;
                        if (n >= 128) break;
                        // first core matrix of this warp in step ks: the previous round's step is done
                        if (g > 0 && n - CUT_WARPS < 32 * ks) ok = umma::mbar_wait(&m->mstep[ks], (g - 1) & 1u) && ok;
                        const int jg = (t & 15) >> 1, hg = 2 * ks + (t & 1), hh = hg * 8 + 2 * kp;
                        float2 x0 = w0[u], x1 = w1[u];
                        if (t < 16) {                          // Ebar rows against the block's largest exponent
                            if (hh < nh) x0 = df_scale(x0, max(xh[hh] - xmax, -1000));
                            if (hh + 1 < nh) x1 = df_scale(x1, max(xh[hh + 1] - xmax, -1000));
                        }
                        float d0[NB], d1[NB];
                        digits_of<NB>(x0.x, x0.y, d0);
                        digits_of<NB>(x1.x, x1.y, d1);
                        unsigned char *dst = sm + (t < 16 ? 0 : GSm<NB>::OFF_B) + (jg * 8 + hg) * 128 + rr * 16 + kp * 4;
#pragma unroll
                        for (int s2 = 0; s2 < NB; s2++)
                            *reinterpret_cast<unsigned *>(dst + s2 * GSm<NB>::PL) = bf16x2(d0[s2], d1[s2]);
                        cut_done(n);
                    }
                }
                // the block's MMAs (the last commit completes after all earlier ones)
                ok = umma::mbar_wait(&m->mstep[3], (gs.nround - 1) & 1u) && ok;
                umma::fence_after();
                ok = __syncthreads_and(ok);
                tick(2);
                if (!ok) break;
                // read-out by all warps: lane half 0 holds level beta + 2, half 1 level beta + 3
                const int qd = warp & 3, hl = qd >> 1, j = 32 * (qd & 1) + lane;
                const uint32_t lane_base = (uint32_t)(32 * qd) << 16;
                const int sc = max(xmax - xr, -1000);
                float2 part[NCOL];
#pragma unroll
                for (int c = 0; c < NCOL; c++) part[c] = make_float2(0.f, 0.f);
#pragma unroll 1
                for (int beta = NB - 1; beta >= 0; beta -= 2) {   // smallest level first, two blocks per wait
                    const int b2 = beta > 0 ? beta - 1 : beta;
                    const int L = beta + 2 + hl, L2 = b2 + 2 + hl;
                    uint32_t rv[NCOL], rv2[NCOL];
                    umma::tmem_ld_nowait(m->tmem + lane_base + 64 * beta + c0, rv);
                    umma::tmem_ld_nowait(m->tmem + lane_base + 64 * b2 + c0, rv2);
                    umma::tmem_wait_ld();
                    if (L <= NB + 1) {
                        const float w = scalbnf(1.0f, -7 * L + sc);
#pragma unroll
                        for (int c = 0; c < NCOL; c++) two_sum_acc(part[c], __uint_as_float(rv[c]), w);
                    }
                    if (b2 != beta && L2 <= NB + 1) {
                        const float w = scalbnf(1.0f, -7 * L2 + sc);
#pragma unroll
                        for (int c = 0; c < NCOL; c++) two_sum_acc(part[c], __uint_as_float(rv2[c]), w);
                    }
                }
                umma::fence_before();
                combine_halves(accs, part, hl, c0, j);
                tick(3);
            }
        }
        if (!ok) {
            if (tid == 0) {
                atomicExch(a.err, 1);
                for (int k = 0; k < 4; k++) umma::mbar_wait(&m->mstep[k], (gs.nround - 1) & 1u, 1000000000ull);
            }
            return false;
        }
    }
    if (row < 64)
#pragma unroll
        for (int c = 0; c < NCOL; c++) out[row * 64 + c0 + c] = df_scale(accs[(c0 + c) * 64 + row], xr);
    for (int q = 0; q < 4; q++) trace_put(tr, tidx, TR_P0 + q, tdur[q]);
    return true;
}

template <int NB>
__global__ void __launch_bounds__(NT, 1) gradP_umma_kernel(FastBwdArgs args) {
    extern __shared__ __align__(1024) unsigned char sm[];
    Misc *m = reinterpret_cast<Misc *>(sm + GSm<NB>::OFF_MISC);
    FastBwdArgs *a = reinterpret_cast<FastBwdArgs *>(sm + GSm<NB>::OFF_ARGS);
    stage(a, &args);
    tmem_setup(m);
    GState gs;
    gradP_task<NB>(*a, blockIdx.x, blockIdx.y, sm, m, gs);
    tmem_teardown(m);
}

// persistent dlnL/dP over (gene, pair, chunk) tasks (independent; heaviest first)
template <int NB>
__global__ void __launch_bounds__(NT, 1) gradP_persist_kernel(const FastBwdArgs *__restrict__ genes,
                                                              const Task *__restrict__ tasks, int ntask,
                                                              unsigned *ctl, unsigned long long *trace) {
    extern __shared__ __align__(1024) unsigned char sm[];
    Misc *m = reinterpret_cast<Misc *>(sm + GSm<NB>::OFF_MISC);
    FastBwdArgs *a = reinterpret_cast<FastBwdArgs *>(sm + GSm<NB>::OFF_ARGS);
    tmem_setup(m);
    GState gs;
    for (;;) {
        const int idx = claim(ctl + CTL_GRADP, m);
        if (idx >= ntask) break;
        trace_put(trace, idx, TR_CLAIM, umma::global_ns());
        const Task t = tasks[idx];
        stage(a, genes + t.gene);
        __syncthreads();
        trace_put(trace, idx, TR_READY, umma::global_ns());
        if (!gradP_task<NB>(*a, t.item, t.tile, sm, m, gs, trace, idx)) break;
        __syncthreads();
        trace_put(trace, idx, TR_END, umma::global_ns());
        trace_put(trace, idx, TR_SM, smid());
    }
    tmem_teardown(m);
}

template <int NS>
cudaError_t init_umma_ns() {
    const void *fu[] = {(const void *)prune_umma_kernel<NS>, (const void *)bwd_umma_kernel<NS>,
                        (const void *)prune_persist_kernel<NS>, (const void *)bwd_persist_kernel<NS>};
    for (const void *f : fu) {
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, USm<NS>::BYTES);
        if (e != cudaSuccess) return e;
    }
    const void *fg[] = {(const void *)gradP_umma_kernel<NS>, (const void *)gradP_persist_kernel<NS>};
    for (const void *f : fg) {
        cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, GSm<NS>::BYTES);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
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

#define GB_NS_SWITCH(ns, CALL)          \
    switch (ns) {                       \
        case 4: CALL(4); break;         \
        case 5: CALL(5); break;         \
        case 6: CALL(6); break;         \
        case 7: CALL(7); break;         \
        case 8: CALL(8); break;         \
    }

void launch_prune_umma(const FastFwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st) {
    dim3 grid(ntile, nitems);
#define L_(n) prune_umma_kernel<n><<<grid, NT, USm<n>::BYTES, st>>>(a)
    GB_NS_SWITCH(ns, L_)
#undef L_
}

void launch_bwd_umma(const FastBwdArgs &a, int ns, int nitems, int ntile, cudaStream_t st) {
    dim3 grid(ntile, nitems);
#define L_(n) bwd_umma_kernel<n><<<grid, NT, USm<n>::BYTES, st>>>(a)
    GB_NS_SWITCH(ns, L_)
#undef L_
}

void launch_gradP_umma(const FastBwdArgs &a, int ns, int npair, cudaStream_t st) {
    dim3 grid(npair, a.nchunk);
#define L_(n) gradP_umma_kernel<n><<<grid, NT, GSm<n>::BYTES, st>>>(a)
    GB_NS_SWITCH(ns, L_)
#undef L_
}

void launch_prune_persist(const FastFwdArgs *genes, const Task *tasks, int ntask, unsigned *ctl, int ns,
                          int nblock, unsigned long long *trace, cudaStream_t st) {
    if (ntask <= 0) return;
    const int g = ntask < nblock ? ntask : nblock;
#define L_(n) prune_persist_kernel<n><<<g, NT, USm<n>::BYTES, st>>>(genes, tasks, ntask, ctl, trace)
    GB_NS_SWITCH(ns, L_)
#undef L_
}

void launch_bwd_persist(const FastBwdArgs *genes, const Task *tasks, int ntask, unsigned *ctl, int ns,
                        int nblock, unsigned long long *trace, cudaStream_t st) {
    if (ntask <= 0) return;
    const int g = ntask < nblock ? ntask : nblock;
#define L_(n) bwd_persist_kernel<n><<<g, NT, USm<n>::BYTES, st>>>(genes, tasks, ntask, ctl, trace)
    GB_NS_SWITCH(ns, L_)
#undef L_
}

void launch_gradP_persist(const FastBwdArgs *genes, const Task *tasks, int ntask, unsigned *ctl, int ns,
                          int nblock, unsigned long long *trace, cudaStream_t st) {
    if (ntask <= 0) return;
    const int g = ntask < nblock ? ntask : nblock;
#define L_(n) gradP_persist_kernel<n><<<g, NT, GSm<n>::BYTES, st>>>(genes, tasks, ntask, ctl, trace)
    GB_NS_SWITCH(ns, L_)
#undef L_
}

namespace {
__global__ void bump_kernel(unsigned *ctl) {
    ctl[CTL_EPOCH] += 1u;
    ctl[CTL_FWD] = 0u;
    ctl[CTL_BWD] = 0u;
    ctl[CTL_GRADP] = 0u;
}
}  // namespace

void launch_bump(unsigned *ctl, cudaStream_t st) { bump_kernel<<<1, 1, 0, st>>>(ctl); }

}  // namespace gb
