// Batch kernel, layout variant set 1 (see batch_body.cuh).
#include "batch_body.cuh"

namespace hg {

HG_BATCH_VARIANT_ENTRY_POINTS(1)

}  // namespace hg
