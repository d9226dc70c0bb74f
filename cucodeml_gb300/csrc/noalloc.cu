// gb_lnL_noalloc: the FP64 lnL evaluation (P(t), pruning levels, mixture) for
// callers that cannot allocate device memory.
//
// Who needs it: a caller whose device memory belongs to someone else -- a
// host application that hands every byte of the GPU to its own pool or
// arena and forbids other allocations, or a latency-sensitive caller that
// cannot afford cudaMalloc/cudaFree, which synchronise the whole device and
// stall its other streams.  Such a caller owns its inputs and outputs (device
// buffers it already has); everything this evaluation needs besides them
// (transition matrices, conditional likelihoods, scale factors, the launch
// schedule) lives in one file-scope device array, g_noalloc_scratch, of
// GB_NOALLOC_SCRATCH_BYTES.  That array is part of the library's device image:
// every GPU that loads the library holds it until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the
// array's device address with cudaGetSymbolAddress and sets the kernels'
// attributes, and caches both for the rest of the process: do not use this
// entry point across a cudaDeviceReset.  No call may be made while its stream
// is being captured into a CUDA graph (it synchronises the stream and uploads
// a host-side schedule that the next call overwrites); such a call returns
// GB_ERR_STATE.  Calls share the array and leave their contents in it; each
// call clears what must start at zero.  Two calls whose work overlaps on the
// GPU race on the array.
//
// Codon ids are checked on the device before any kernel reads them: an id
// outside 0..60 (codeml's ambiguity codes, or any stray byte) is replaced by
// 0 in the scratch copy, flagged, and the call returns GB_ERR_ARG without
// touching the caller's outputs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "handle.h"

namespace {

__device__ __align__(256) unsigned char g_noalloc_scratch[GB_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxNode = 256;
constexpr int kMaxDev = 64;

struct Sched {   // host-side launch schedule, built in static storage
    int ns, nn, root, npatt, npad, ntile, H;
    int nson[kMaxNode], sons[kMaxNode * gb::MAXC], height[kMaxNode], dirty[kMaxNode];
    int scale[kMaxNode], order[kMaxNode], d[kMaxNode], label[kMaxNode];
    int nscale, nslot, nsslot, npair, nitems;
    int slot_of[kMaxNode * 4], sslot_of[kMaxNode * 4], pair_of[kMaxNode * 3];
    gb::PairDesc pairs[kMaxNode * 3];
    int scale_list[4 * kMaxNode];
    gb::Item items[kMaxNode * 4];
    int level_off[kMaxNode + 1];
};

std::mutex g_mu;             // one call at a time on the host side
Sched g_s;
void *g_scratch[kMaxDev] = {};

int setup_device(int dev, unsigned char **out) {
    if (dev < 0 || dev >= kMaxDev) return gb::fail(GB_ERR_ARG, "gb_lnL_noalloc: device ordinal out of range");
    if (!g_scratch[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return gb::cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        e = gb::init_fp64_kernels();
        if (e != cudaSuccess) return gb::cuda_fail(e, "kernel attributes");
        g_scratch[dev] = p;
    }
    *out = static_cast<unsigned char *>(g_scratch[dev]);
    return 0;
}

int build(Sched &s, int ns, int nn, int root, const int *father, const int *label, const char *node_scale,
          int npatt) {
    using gb::MAXC;
    if (ns < 3 || nn < ns + 1 || nn > kMaxNode || npatt < 1 || !father || !label)
        return gb::fail(GB_ERR_ARG, "gb_lnL_noalloc: sizes out of range (at most 256 nodes)");
    if (root < ns || root >= nn || father[root] != -1)
        return gb::fail(GB_ERR_ARG, "gb_lnL_noalloc: root must be an internal node with father -1");
    s.ns = ns; s.nn = nn; s.root = root; s.npatt = npatt;
    s.npad = (npatt + gb::TILE64 - 1) / gb::TILE64 * gb::TILE64;
    s.ntile = s.npad / gb::TILE64;
    for (int n = 0; n < nn; n++) { s.nson[n] = 0; s.height[n] = 0; s.dirty[n] = 0; s.scale[n] = 0; s.label[n] = 0; }
    for (int n = 0; n < nn; n++) {
        if (n == root) continue;
        int f = father[n];
        if (f < ns || f >= nn || s.nson[f] >= MAXC) return gb::fail(GB_ERR_ARG, "gb_lnL_noalloc: bad father array");
        if (label[n] != 0 && label[n] != 1) return gb::fail(GB_ERR_ARG, "gb_lnL_noalloc: labels must be 0 or 1");
        s.sons[f * MAXC + s.nson[f]++] = n;
        s.label[n] = label[n];
    }
    for (int n = 0; n < nn; n++)
        if ((n < ns && s.nson[n]) || (n >= ns && s.nson[n] < 2))
            return gb::fail(GB_ERR_ARG, "gb_lnL_noalloc: tips must be nodes 0..ns-1, internal nodes need 2-3 sons");
    int cnt = 0;
    s.order[cnt++] = root;
    for (int i = 0; i < cnt; i++)
        for (int k = 0; k < s.nson[s.order[i]]; k++) {
            if (cnt >= nn) return gb::fail(GB_ERR_ARG, "gb_lnL_noalloc: not a tree");
            s.order[cnt++] = s.sons[s.order[i] * MAXC + k];
        }
    if (cnt != nn) return gb::fail(GB_ERR_ARG, "gb_lnL_noalloc: tree is not connected");
    for (int i = nn - 1; i >= 0; i--) {
        int a = s.order[i];
        int tips = a < ns ? 1 : 0;
        for (int k = 0; k < s.nson[a]; k++) {
            int c = s.sons[a * MAXC + k];
            s.height[a] = std::max(s.height[a], s.height[c] + 1);
            if (s.label[c] == 1 || s.dirty[c]) s.dirty[a] = 1;
            tips += s.d[c];
        }
        // scaled nodes: given, or codeml's rule (more than 15 tips since the last scaled node)
        if (node_scale) s.scale[a] = (a >= ns && a != root && node_scale[a]) ? 1 : 0;
        else if (a >= ns && a != root && tips > 15) { s.scale[a] = 1; tips = 1; }
        s.d[a] = tips;
    }
    s.nscale = 0;
    for (int n = 0; n < nn; n++) s.nscale += s.scale[n];
    auto ncls = [&](int a) { return (s.dirty[a] || a == root) ? 4 : 2; };
    auto cls_of = [&](int c2, int c) { return (s.dirty[c2] || c2 == root) ? c : (c & 1); };
    s.nslot = s.nsslot = 0;
    for (int i = 0; i < nn * 4; i++) { s.slot_of[i] = -1; s.sslot_of[i] = -1; }
    for (int a = ns; a < nn; a++)
        for (int c = 0; c < ncls(a); c++) {
            s.slot_of[a * 4 + c] = s.nslot++;
            if (s.scale[a]) s.sslot_of[a * 4 + c] = s.nsslot++;
        }
    s.npair = 0;
    for (int i = 0; i < nn * 3; i++) s.pair_of[i] = -1;
    for (int n = 0; n < nn; n++) {
        if (n == root) continue;
        for (int w = 0; w < (s.label[n] ? 3 : 2); w++) {
            s.pair_of[n * 3 + w] = s.npair;
            s.pairs[s.npair++] = gb::PairDesc{n, w};
        }
    }
    for (int c = 0; c < 4; c++) {
        int k = 0;
        for (int b = 0; b < nn; b++)
            if (s.scale[b]) s.scale_list[c * s.nscale + k++] = s.sslot_of[b * 4 + cls_of(b, c)];
    }
    s.H = s.height[root];
    s.nitems = 0;
    for (int L = 1; L <= s.H; L++) {
        s.level_off[L - 1] = s.nitems;
        for (int a = ns; a < nn; a++) {
            if (s.height[a] != L) continue;
            for (int c = 0; c < ncls(a); c++) {
                gb::Item &it = s.items[s.nitems++];
                it.node = a; it.cls = c; it.slot = s.slot_of[a * 4 + c];
                it.nchild = s.nson[a];
                for (int k = 0; k < MAXC; k++) { it.child[k] = -1; it.cslot[k] = -1; it.pidx[k] = -1; }
                for (int k = 0; k < it.nchild; k++) {
                    int c2 = s.sons[a * MAXC + k];
                    it.child[k] = c2;
                    it.cslot[k] = c2 < ns ? -1 : s.slot_of[c2 * 4 + cls_of(c2, c)];
                    int w = s.label[c2] == 0 ? (c & 1) : (c <= 1 ? c : 2);
                    it.pidx[k] = s.pair_of[c2 * 3 + w];
                }
                it.sslot = s.scale[a] ? s.sslot_of[a * 4 + c] : -1;
                it.is_root = a == root;
                it.eslot = it.slot * MAXC;
            }
        }
    }
    s.level_off[s.H] = s.nitems;
    return 0;
}

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

// Codon ids of the scratch copy of z (ns rows of npad, npatt used): an id
// of 61 or more would index past the 61 rows of a transition matrix in the
// pruning kernels, so it is replaced by 0 and flagged before they run.
__global__ void noalloc_check_z(unsigned char *z, int ns, int npad, int npatt, unsigned *bad) {
    const size_t n = (size_t)ns * npad;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if ((int)(i % npad) >= npatt) continue;
        if (z[i] >= 61) {
            z[i] = 0;
            atomicOr(bad, 1u);
        }
    }
}

}  // namespace

extern "C" int gb_lnL_noalloc(int ns, int nnode, int root, const int *father, const int *label,
                              const char *node_scale, int npatt, const unsigned char *d_z,
                              const double *d_fpatt, const double *d_pi, const double *d_model,
                              const double *d_blength, double *d_neg_lnL, double *d_fhK, void *stream) {
    using namespace gb;
    if (!d_z || !d_fpatt || !d_pi || !d_model || !d_blength || !d_neg_lnL)
        return fail(GB_ERR_ARG, "gb_lnL_noalloc: null device pointer");
    {
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap));
        if (cap != cudaStreamCaptureStatusNone)
            return fail(GB_ERR_STATE, "gb_lnL_noalloc: not callable during stream capture");
    }
    std::lock_guard<std::mutex> lock(g_mu);
    int dev = 0;
    CK(cudaGetDevice(&dev));
    unsigned char *base = nullptr;
    int rc = setup_device(dev, &base);
    if (rc) return rc;
    Sched &s = g_s;
    rc = build(s, ns, nnode, root, father, label, node_scale, npatt);
    if (rc) return rc;

    // carve the scratch array
    const size_t npad = s.npad;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off = align256(off + bytes); return o; };
    const size_t o_items = take(sizeof(Item) * s.nitems);
    const size_t o_pairs = take(sizeof(PairDesc) * s.npair);
    const size_t o_label = take(sizeof(int) * s.nn);
    const size_t o_slist = take(sizeof(int) * 4 * std::max(s.nscale, 1));
    const size_t o_z = take((size_t)s.ns * npad);
    const size_t o_Pt = take(sizeof(double) * (size_t)s.npair * 64 * 64);
    const size_t o_conP = take(sizeof(double) * (size_t)s.nslot * npad * 64);
    const size_t o_scaleF = take(sizeof(double) * (size_t)std::max(s.nsslot, 1) * npad);
    const size_t o_fbar = take(sizeof(double) * 4 * npad);
    const size_t o_ssum = take(sizeof(double) * 4 * npad);
    const size_t o_fhK = take(sizeof(double) * 4 * npad);
    const size_t o_part = take(sizeof(double) * (npad / 256 + 2));
    const size_t o_ticket = take(sizeof(unsigned));
    const size_t o_bad = take(sizeof(unsigned));
    const size_t o_lnL = take(sizeof(double));
    if (off > (size_t)GB_NOALLOC_SCRATCH_BYTES) {
        char msg[200];
        snprintf(msg, sizeof msg,
                 "gb_lnL_noalloc: this problem needs %zu bytes of scratch, the limit is %u "
                 "(GB_NOALLOC_SCRATCH_BYTES); use gb_create + gb_eval_uvr",
                 off, (unsigned)GB_NOALLOC_SCRATCH_BYTES);
        return fail(GB_ERR_ARG, msg);
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    Item *items = reinterpret_cast<Item *>(base + o_items);
    PairDesc *pairs = reinterpret_cast<PairDesc *>(base + o_pairs);
    int *lab = reinterpret_cast<int *>(base + o_label);
    int *slist = reinterpret_cast<int *>(base + o_slist);
    unsigned char *z = base + o_z;
    double *Pt = reinterpret_cast<double *>(base + o_Pt);
    double *conP = reinterpret_cast<double *>(base + o_conP);
    double *scaleF = reinterpret_cast<double *>(base + o_scaleF);
    double *fbar = reinterpret_cast<double *>(base + o_fbar);
    double *ssum = reinterpret_cast<double *>(base + o_ssum);
    double *fhK = reinterpret_cast<double *>(base + o_fhK);
    double *part = reinterpret_cast<double *>(base + o_part);
    unsigned *ticket = reinterpret_cast<unsigned *>(base + o_ticket);
    unsigned *bad = reinterpret_cast<unsigned *>(base + o_bad);
    double *lnL = reinterpret_cast<double *>(base + o_lnL);

    CK(cudaMemcpyAsync(items, s.items, sizeof(Item) * s.nitems, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(pairs, s.pairs, sizeof(PairDesc) * s.npair, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(lab, s.label, sizeof(int) * s.nn, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(slist, s.scale_list, sizeof(int) * 4 * std::max(s.nscale, 1), cudaMemcpyHostToDevice, st));
    // zero what must start at zero: the padded tail of z and the reduction ticket
    CK(cudaMemsetAsync(z, 0, (size_t)s.ns * npad, st));
    CK(cudaMemcpy2DAsync(z, npad, d_z, s.npatt, s.npatt, s.ns, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemsetAsync(ticket, 0, sizeof(unsigned), st));
    CK(cudaMemsetAsync(bad, 0, sizeof(unsigned), st));
    noalloc_check_z<<<std::min<size_t>(1024, ((size_t)s.ns * npad + 255) / 256), 256, 0, st>>>(
        z, s.ns, (int)npad, s.npatt, bad);
    const DevParams *prm = reinterpret_cast<const DevParams *>(d_model);
    launch_pmat_fp64(pairs, s.npair, lab, d_blength, prm, Pt, st);
    for (int L = 0; L < s.H; L++) {
        int n = s.level_off[L + 1] - s.level_off[L];
        if (n)
            launch_prune_fp64(items + s.level_off[L], n, s.ntile, s.npad, z, Pt, conP, nullptr, scaleF,
                              slist, s.nscale, d_pi, fbar, ssum, fhK, st);
    }
    launch_mix(fhK, d_fpatt, prm, s.npatt, s.npad, s.nscale, nullptr, nullptr, part, ticket, lnL, st);
    unsigned flagged = 0;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(&flagged, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (flagged) return fail(GB_ERR_ARG, "gb_lnL_noalloc: codon ids must be 0..60 (sense codons)");
    CK(cudaMemcpyAsync(d_neg_lnL, lnL, sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (d_fhK)
        CK(cudaMemcpy2DAsync(d_fhK, sizeof(double) * s.npatt, fhK, sizeof(double) * npad,
                             sizeof(double) * s.npatt, 4, cudaMemcpyDeviceToDevice, st));
    CK(cudaStreamSynchronize(st));
    return GB_OK;
}
