// Internal types shared by the host runtime (runtime.cu) and the kernels.
//
// Data layout in HBM (per handle):
//   Pt     [npair][64][64]   FP64 transposed transition matrices, one per unique
//                            (branch, omega) pair: Pt[k][j] = P(t)[j][k], zero
//                            padded beyond 61 (k = child state, j = parent state).
//   conP   [nslot][npad][64] FP64 conditional likelihoods per (node, class) slot,
//                            pattern-major, 64 states per row (61 used).
//   E      [nslot*3][npad][64] per-edge messages P.L (kept for the adjoint).
//   scaleF [nsslot][npad]    log scale factors of scaled (node, class) slots.
//   fbar / ssum / fhK [4][npad]  root f~ (floored), summed scale logs, codeml's fhK.
//
// A "slot" is one (internal node, site class) pair that is actually computed.
// Classes 0 and 1 are computed at every internal node; classes 2a/2b only at
// "dirty" nodes, those with a foreground-labelled branch at or below them: at
// every other node class 2a equals class 0 and 2b equals class 1 exactly
// (same omega on every branch below, Set_UVR_BranchSite codeml.c:2545-2568).
#pragma once

#include <cstdint>

namespace gb {

constexpr int MAXC = 3;       // children per internal node (binary tree, trifurcating root)
constexpr int TILE64 = 32;    // patterns per CTA tile in the FP64 kernels

struct Item {                 // one (internal node, class) slot
    int node, cls, slot;      // output slot (conP row block)
    int nchild;
    int child[MAXC];          // child node id
    int cslot[MAXC];          // child's conP slot, -1 for a tip
    int pidx[MAXC];           // transition matrix (pair) of the edge under this class
    int sslot;                // scale slot, -1 if the node is not scaled
    int is_root;
    int eslot;                // first of nchild E slots (slot * MAXC)
};

struct PairDesc {             // one (branch, omega) transition matrix
    int node;                 // branch above this node
    int w;                    // omega index 0 (w0), 1 (w1 = 1), 2 (w2)
};

struct DevParams {            // uploaded per evaluation
    double U[3][61 * 61];
    double V[3][61 * 61];
    double Root[3][61];
    double qf[2];
    double freqK[4];
    int sym;                   // V[m][k] = U[k][m] pi_k (symmetrised eigenproblem): P from its symmetric part;
                               // after the GB_MODEL_DOUBLES of the no-alloc model block, never read from one
};

// ---- kernel launchers (k_fp64.cu) ----
cudaError_t init_fp64_kernels();   // function attributes; call before any capture
// pi (nullable): the codon frequencies of a model whose U and V come from the
// symmetrised eigenproblem (V[m][k] = U[k][m] pi_k): P is then formed from its
// symmetric part S = U diag(e) U^T at about half the FP64 work
void launch_pmat_fp64(const PairDesc *pairs, int npair, const int *label, const double *tnode,
                      const DevParams *prm, double *Pt, cudaStream_t st, const double *pi = nullptr);
void launch_prune_fp64(const Item *items, int nitems, int ntile, int npad, const unsigned char *z,
                       const double *Pt, double *conP, double *E, double *scaleF,
                       const int *scale_list, int nscale, const double *pi, double *fbar,
                       double *ssum, double *fhK, cudaStream_t st, const unsigned char *amb = nullptr);
void launch_mix(const double *fhK, const double *fpatt, const DevParams *prm, int npatt, int npad,
                int nscale, double *lnf, double *post, double *partial, unsigned *ticket,
                double *out, cudaStream_t st, const double *fbar = nullptr, float2 *groot = nullptr);

}  // namespace gb
