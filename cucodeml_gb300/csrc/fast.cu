// Split-precision path (GB_PREC_FAST).  Placeholder until the kernels land:
// the call fails loudly rather than falling back to another path.
#include "handle.h"

namespace gb {

struct FastState {};

void fast_free(FastState *f) { delete f; }

int fast_eval(gb_handle *h, const Derived *D, const double *blength, double *neg_lnL, gb_grad *grad,
              double *fhK, double *lnf, gb_stats *stats) {
    (void)h; (void)D; (void)blength; (void)neg_lnL; (void)grad; (void)fhK; (void)lnf; (void)stats;
    return fail(GB_ERR_STATE, "GB_PREC_FAST is not available in this build");
}

int fast_replay(gb_handle *, int, int, double *) {
    return fail(GB_ERR_STATE, "GB_PREC_FAST is not available in this build");
}

int fast_profile(gb_handle *, int, int, double *, int *) {
    return fail(GB_ERR_STATE, "GB_PREC_FAST is not available in this build");
}

}  // namespace gb
