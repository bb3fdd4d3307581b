// Entry points of subsystems that are not built yet report
// GBFFT_ERR_UNSUPPORTED so the C ABI stays complete.
#include "gbfft.h"
#include "plan_internal.h"

namespace gbfft {
int build_split_plan(gbfft_plan*) { return GBFFT_ERR_UNSUPPORTED; }
}  // namespace gbfft
