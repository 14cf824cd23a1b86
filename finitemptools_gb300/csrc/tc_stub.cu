// Placeholder for the tensor-core (mixed precision) path until it lands.
#include "internal.h"

namespace fmpt {
int op_tc_prepare(fmpt_op* op) {
  return set_error(op->h, FMPT_ERR_UNSUPPORTED, "mixed precision not built yet");
}
int op_tc_apply(fmpt_op* op, const double*, double*) {
  return set_error(op->h, FMPT_ERR_UNSUPPORTED, "mixed precision not built yet");
}
void op_tc_free(fmpt_op*) {}
}  // namespace fmpt
