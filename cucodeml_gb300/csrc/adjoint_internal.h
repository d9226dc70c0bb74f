// Adjoint structures shared by the FP64 adjoint (adjoint.cu) and the
// split-precision adjoint (k_fast_bwd.cu, fast.cu).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "gbcodeml.h"
#include "internal.h"
#include "model.h"

struct gb_handle;

namespace gb {

constexpr int GCHUNK = 512;   // patterns per partial of dlnL/dP (FP64 kernel)
constexpr int GCHUNK_FAST = 2048;   // default of the split-precision kernels (measured fastest on a
                                    // single 64 x 5000 alignment and on a 512-gene batch; a single
                                    // small alignment halves it while its tasks are too few)
// dP/dt buffer: derivative matrices V dQ U at 0..4 (kappa for w0, w1, w2;
// omega for w0, w2), the inverse-difference tables of w0, w1, w2 at 5..7, and
// the omega derivative of slot 1 at 8 (branch-site model B's free w1; zero
// under model A, where w1 = 1)
constexpr int DM_MATS = 9;
constexpr int DM_RB = 4;      // dP/dt kernel: row blocks per derivative matrix
constexpr int DM_NDER = 6;    // derivative matrices formed
constexpr int DM_BLOCKS = DM_NDER * DM_RB + 3;
constexpr int DM_OMEGA1 = 8;  // index of the slot-1 omega derivative
constexpr int UVDF_DM = 3 * 2 * 61 * 64;   // offset of the double-float tables in d_UVdf

struct BItem {                // backward work: (node, class family) of one level
    int node, ncls, is_root, nchild;
    int cls[2], pslot[2], sslot[2];
    int eslot[2];             // first E / Ebar row block of the node's class k (FP64 path)
    int pidx[MAXC][2];        // pair of edge i under parent class k
    int tslot[MAXC][2];       // child slot receiving the adjoint (-1: tip)
    int child[MAXC];          // child node of edge i
};

struct Contrib {              // one (parent slot, child) term of dlnL/dP for a pair
    int ebar;                 // index into Ebar (= parent slot * MAXC + child index)
    int tslot;                // child conP slot, or -1 for a tip
    int tip;                  // tip node when tslot < 0
};

struct GradParams {
    double dQk[3][61 * 61];
    double dQw[3][61 * 61];
};

struct AdjointState {
    std::vector<BItem> bitems;
    std::vector<int> blevel_off;     // top-down order of levels
    std::vector<Contrib> contrib;
    std::vector<int> coff;
    int nchunk = 1, nfreq_blocks = 1;
    int gchunk = GCHUNK;             // patterns per dlnL/dP partial
    BItem *d_bitems = nullptr;
    Contrib *d_contrib = nullptr;
    int *d_coff = nullptr;
    double *d_Ebar = nullptr, *d_Abar = nullptr, *d_Gpart = nullptr, *d_Dm = nullptr;
    double *d_pout = nullptr, *d_fpart = nullptr;
    float2 *d_UVdf = nullptr;        // split precision, double-float: [3][2][61][64] V^T and U, then (at
                                     // UVDF_DM) [DM_MATS][64][64] the dP/dt and inverse-difference tables
    GradParams *d_gp = nullptr, *h_gp = nullptr;
    double *h_pout = nullptr, *h_fpart = nullptr;
    cudaGraphExec_t graph = nullptr;
    int graph_kernels = 0;
    double d_omega1 = 0;             // d(-lnL)/d w1 of the last chain rule (model B)
    // checkpointed adjoint (FP64, gb_tune GB_TUNE_CHECKPOINT): conditional
    // likelihoods kept at every internal node, the edge messages E and Ebar
    // of one tree level at a time, recomputed level by level in the reverse
    // sweep; per level: the forward items to recompute (E rows level-local),
    // and the pairs whose dlnL/dP that level completes
    bool ckpt = false;
    int ckpt_rows = 0;               // E / Ebar slots of the widest level
    std::vector<Item> ritems;        // forward items in the adjoint's level order
    std::vector<int> rlevel_off;
    std::vector<int> plist, plevel_off;
    Item *d_ritems = nullptr;
    int *d_plist = nullptr;
};

int adjoint_init(gb_handle *h);               // host structures and device buffers
void launch_dmat(gb_handle *h);
void launch_gradH(gb_handle *h);
void launch_gradH_df(gb_handle *h);      // split-precision path: double-float products
void launch_freq(gb_handle *h, int nscale);
void adjoint_chain(gb_handle *h, const Derived *D, const double *blength, gb_grad *grad);
int adjoint_fetch(gb_handle *h);              // D2H of per-pair and class-weight sums (async)
// the FP64 gradient kernels on explicit buffers (clade models): attributes
// (before any capture), dP/dt matrices of one parameter block, one backward
// level, dlnL/dP partials of every pair, per-pair sums (dt', kappa, omega of
// the pair's eigen slot), class-weight sums ((npatt + 255) / 256 blocks of 4)
cudaError_t init_fp64_adjoint_kernels();
void launch_dmat_fp64(const DevParams *prm, const GradParams *gp, double *Dm, cudaStream_t st);
void launch_bwd_level_fp64(const BItem *bitems, int nitems, int ntile, int npad, const double *Pt, const double *E,
                           double *Ebar, double *Abar, const double *scaleF, const double *fpatt, const double *post,
                           const double *fbar, const double *pi, cudaStream_t st);
void launch_gradP_fp64(const Contrib *contrib, const int *coff, int npair, int nchunk, int npatt, int npad,
                       const double *Ebar, const double *conP, const unsigned char *z, double *Gpart,
                       const unsigned char *amb, cudaStream_t st);
void launch_gradH_fp64(const PairDesc *pairs, int npair, const int *label, const double *tnode, const DevParams *prm,
                       const double *Gpart, int nchunk, const double *Dm, double *pout, cudaStream_t st);
void launch_freq_fp64(const double *fhK, const double *lnf, const double *fpatt, int npatt, int npad, int nscale,
                      double *fpart, cudaStream_t st);

}  // namespace gb
