// ocn_mixed.cu -- mixed-precision long-range term (split-BF16 tcgen05 u2
// contractions, FP32 k-mesh transform).  Placeholder until the tensor-core path
// lands: a mixed-precision context reports OCN_ERR_UNSUPPORTED instead of
// silently running another path.
#include "ocn_internal.h"

namespace ocn {

struct MixedLR {
  int dummy = 0;
};

int mixed_init(ocn_ctx* c) {
  c->mixed = new MixedLR();
  return OCN_OK;
}

int mixed_free(ocn_ctx* c) {
  delete c->mixed;
  c->mixed = nullptr;
  return OCN_OK;
}

int mixed_set_bloch(ocn_ctx* c) { return OCN_OK; }

int lr_apply_mixed(ocn_ctx* c, const double*, const double*) {
  return set_err(c, OCN_ERR_UNSUPPORTED, "mixed-precision long-range path not built");
}

}  // namespace ocn
